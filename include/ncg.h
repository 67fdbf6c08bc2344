/*
 * ncg.h — C ABI of the GB300 batched convex narrow phase (GJK + EPA).
 *
 * Every entry point replaces a per-pair function of ncollide3d 0.33 with a
 * batched call over N independent pairs (Isometry3, SupportMap, Isometry3,
 * SupportMap).  Plain pointers and sizes only: no CUDA, torch or C++ types.
 * Functions named *_batch take DEVICE pointers and are asynchronous on the
 * given stream (a cudaStream_t passed as void*, NULL = legacy default stream);
 * functions named *_batch_host take HOST pointers, copy inputs to the device,
 * run, copy results back and return when the results are in host memory.
 *
 * Reference interfaces (paths inside the ncollide repository):
 *   contact    src/query/contact/contact_support_map_support_map.rs:9-30, 38-88
 *   distance   src/query/distance/distance_support_map_support_map.rs:8-53
 *   proximity  src/query/proximity/proximity_support_map_support_map.rs:10-75
 *   closest    src/query/closest_points/closest_points_support_map_support_map.rs:9-67
 *   toi        src/query/time_of_impact/time_of_impact.rs:63-90,
 *              src/query/time_of_impact/time_of_impact_support_map_support_map.rs:10-127
 *   ray cast   src/query/ray/ray_support_map.rs:14-110, src/query/algorithms/gjk.rs:180-194
 *   aabb       src/bounding_volume/aabb_*.rs; broad phase src/pipeline/broad_phase/dbvt_broad_phase.rs
 *   manifold   src/pipeline/narrow_phase/contact_generator/convex_polyhedron_convex_polyhedron_manifold_generator.rs
 * The per-pair arithmetic is gjk::closest_points (src/query/algorithms/gjk.rs:76-177)
 * with VoronoiSimplex (voronoi_simplex3.rs) and EPA (epa3.rs:219-454).
 */
#ifndef NCG_H
#define NCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2: ncg_stats gained n_epa_thread (56 bytes); NCG_TUNE_HULL_STAGE_*, ncg_autotune,
 * ncg_ctx_get_tuning and NCG_EINTERNAL added.
 * 3: ncg_ctx_set_arithmetic (NCG_ARITH_SPLIT, NCG_ARITH_F32), NCG_TUNE_HULL_EPA_WARP and
 * NCG_TUNE_HULL_LOCALITY (NCG_N_TUNE 8), the ConvexHull topology and
 * ncg_manifold_batch_hulls added.
 * ncg_abi_version() returns it. */
#define NCG_ABI_VERSION 3

/* ---- shape kinds: the ncollide3d shapes that implement SupportMap ------- */
enum ncg_shape_kind {
    NCG_BALL = 0,        /* src/shape/ball.rs:29-49        p = {radius}                 */
    NCG_CUBOID = 1,      /* src/shape/cuboid.rs:135-146    p = {hx, hy, hz}             */
    NCG_CAPSULE = 2,     /* src/shape/capsule.rs:72-84     p = {half_height, radius}    */
    NCG_CONE = 3,        /* src/shape/cone.rs:45-67        p = {half_height, radius}    */
    NCG_CYLINDER = 4,    /* src/shape/cylinder.rs:47-63    p = {half_height, radius}    */
    NCG_CONVEX_HULL = 5  /* src/shape/convex.rs:418-423    points[hull_off .. +hull_n]  */
};

/* Isometry3<f32>: unit quaternion (i, j, k, w) — nalgebra's coordinate order —
 * then the translation.  32 bytes so one pose is two 128-bit loads. */
typedef struct ncg_pose {
    float q[4];
    float t[3];
    float pad;
} ncg_pose;

/* One shape record, 32 bytes.  Convex hull vertices live in one flat array of
 * float4 (x, y, z, unused) shared by all hulls; a hull owns the slice
 * [hull_off, hull_off + hull_n) of it.  The arg-max over that slice is
 * ncollide's point_cloud_support_point (first maximum wins). */
typedef struct ncg_shape {
    uint32_t kind;
    uint32_t hull_off;
    uint32_t hull_n;
    uint32_t pad;
    float p[4];
} ncg_shape;

/* query::Contact<f32> (src/query/contact/contact.rs:15-27). */
typedef struct ncg_contact {
    float world1[3];
    float world2[3];
    float normal[3];
    float depth;
} ncg_contact;

/* One batch of pairs.  Pair i is (m1[i], shapes[g1[i]], m2[i], shapes[g2[i]]).
 * init_dir, when not NULL, holds 3 floats per pair: the unit direction the
 * *_with_params functions accept as `init_dir` (GJK warm start). */
typedef struct ncg_batch {
    const ncg_shape* shapes;
    const float* hull_points;   /* 4 floats per vertex, 16-byte aligned */
    uint32_t n_shapes;
    uint32_t pad0;
    uint64_t n_hull_points;
    const ncg_pose* m1;
    const uint32_t* g1;
    const ncg_pose* m2;
    const uint32_t* g2;
    uint64_t n_pairs;
    const float* init_dir;
} ncg_batch;

/* Proximity (src/query/proximity/proximity.rs:4-11), same discriminants. */
enum ncg_proximity { NCG_INTERSECTING = 0, NCG_WITHIN_MARGIN = 1, NCG_DISJOINT = 2 };

/* ClosestPoints (src/query/closest_points/closest_points.rs:8-15). */
enum ncg_closest_points { NCG_CP_INTERSECTING = 0, NCG_CP_WITHIN_MARGIN = 1, NCG_CP_DISJOINT = 2 };

/* Per-pair status bits.  The reference panics or silently returns None in
 * these cases; the batch API never traps and reports them instead. */
#define NCG_STATUS_OK            0u
#define NCG_STATUS_GJK_MAX_ITER  (1u << 0) /* gjk.rs:172-175 iteration cap          */
#define NCG_STATUS_EPA_FAILED    (1u << 1) /* EPA returned None: epa3.rs:278-293,369-372,404,409-413 */
#define NCG_STATUS_EPA_MAX_ITER  (1u << 2) /* epa3.rs:421-424 iteration cap          */
#define NCG_STATUS_EPA_CAPACITY  (1u << 3) /* polytope outgrew the device capacity   */
#define NCG_STATUS_EPA_NO_FACE   (1u << 4) /* reference panics at epa3.rs:325        */
#define NCG_STATUS_DEGENERATE    (1u << 5) /* reference asserts (point_tetrahedron.rs:295) */
#define NCG_STATUS_BAD_INPUT     (1u << 6) /* shape index out of range, bad hull slice */
#define NCG_STATUS_UNSUPPORTED_FEATURE (1u << 7) /* query dispatch: ball centre on a ConvexHull's
                                                    surface needs the hull's face topology */
#define NCG_STATUS_MANIFOLD_FULL (1u << 10) /* manifold: clipping produced more than
                                                    NCG_MANIFOLD_MAX contacts; the first
                                                    NCG_MANIFOLD_MAX are kept */
#define NCG_STATUS_NOT_POLYHEDRA (1u << 9) /* manifold: not a Cuboid pair; the manifold is the
                                              single GJK/EPA contact with unknown features  */
#define NCG_STATUS_EPA_PRECISION_LIMIT (1u << 8) /* NCG_TOL_PRECISE: EPA's expansion would have
                                                    returned None (f32 noise on sliver faces); the
                                                    contact is the best face found so far */

/* query::TOI<f32> (src/query/time_of_impact/time_of_impact.rs:29-42):
 * witnesses and normals in the shapes' local frames; valid when has_toi. */
/* Contact manifolds.  FeatureId (src/shape/feature_id.rs) packed as
 * kind << 28 | id with kind NCG_FEATURE_*; Cuboid ids as in cuboid.rs:148-277. */
enum ncg_feature_kind { NCG_FEATURE_UNKNOWN = 0, NCG_FEATURE_VERTEX = 1, NCG_FEATURE_EDGE = 2,
                        NCG_FEATURE_FACE = 3 };
#define NCG_MANIFOLD_MAX 16
typedef struct ncg_manifold_point {
    float world1[3];
    float world2[3];
    float depth;
    uint32_t feature1, feature2;
} ncg_manifold_point;
/* The contacts ConvexPolyhedronConvexPolyhedronManifoldGenerator::generate_contacts
 * pushes for one pair, all with the pair's normal. */
typedef struct ncg_manifold {
    float normal[3];
    uint32_t n;
    ncg_manifold_point points[NCG_MANIFOLD_MAX];
} ncg_manifold;

typedef struct ncg_toi {
    float toi;
    float witness1[3];
    float witness2[3];
    float normal1[3];
    float normal2[3];
    uint32_t status; /* enum ncg_toi_status */
} ncg_toi;

/* TOIStatus (time_of_impact.rs:7-26), same discriminants. */
enum ncg_toi_status {
    NCG_TOI_OUT_OF_ITERATIONS = 0,
    NCG_TOI_CONVERGED = 1,
    NCG_TOI_FAILED = 2,
    NCG_TOI_PENETRATING = 3
};

/* Return codes. */
#define NCG_OK          0
#define NCG_EINVAL     (-1)  /* bad argument (e.g. margin < 0, NULL required pointer) */
#define NCG_ECUDA      (-2)  /* a CUDA call failed; ncg_last_error() has the text     */
#define NCG_ENOMEM     (-3)
#define NCG_ENOTBUILT  (-4)
#define NCG_EINTERNAL  (-5)  /* a self-check failed (e.g. results depended on tuning) */

/* Tolerance sets.  NCG_TOL_REFERENCE uses the reference's own f32 constants
 * (eps = f32::EPSILON: gjk eps_tol = 10 eps, eps_rel = sqrt(eps_tol), EPA
 * termination 100 eps).  NCG_TOL_PRECISE tightens the termination tests so
 * that results land within 1e-5 relative of the f64 reference. */
enum ncg_tolerance { NCG_TOL_REFERENCE = 0, NCG_TOL_PRECISE = 1 };

/* Arithmetic of GJK, EPA and the query wrappers (contact, distance,
 * proximity, closest points, the manifold's contact query).
 * NCG_ARITH_SPLIT (default): support mapping, CSO points and EPA's expansion
 *   in f32; the Voronoi-simplex sub-solve, GJK's bounds and EPA's face
 *   normals, distances and termination in double-word arithmetic (~48-bit
 *   significand on the FP32 pipes); EPA's queue pops equal distances first
 *   in, first out.
 * NCG_ARITH_F32: the reference's f32 path as the reference computes it
 *   (N = f32 throughout: the f32 sub-solve and constants, and Rust
 *   BinaryHeap's order among equal EPA distances), for callers that need its
 *   results bit for bit rather than the split's FP64-class accuracy. */
enum ncg_arithmetic { NCG_ARITH_SPLIT = 0, NCG_ARITH_F32 = 1 };

/* Pair dispatch of ncg_contact_batch.
 * NCG_DISPATCH_SUPPORT_MAP: every pair through contact_support_map_support_map
 *   (GJK, then EPA) — the (&dyn SupportMap, &dyn SupportMap) semantics.
 * NCG_DISPATCH_QUERY: query::contact's routing (contact_shape_shape.rs:10-47):
 *   Ball-Ball by contact_ball_ball, Ball against Cuboid or ConvexHull by
 *   contact_ball_convex_polyhedron (point projection), every other pair by
 *   contact_support_map_support_map.  `out_dir` then holds the contact normal
 *   (zeros for no contact) for the first two routes. */
enum ncg_dispatch { NCG_DISPATCH_SUPPORT_MAP = 0, NCG_DISPATCH_QUERY = 1 };

/* Warm-start sources for the first GJK direction. */
enum ncg_warm_start {
    NCG_WARM_NONE = 0,      /* reference default: normalize(t2 - t1) (contact/proximity) */
    NCG_WARM_INIT_DIR = 1,  /* batch->init_dir (the *_with_params init_dir argument); an
                               all-zero entry means None for that pair                    */
    NCG_WARM_MLP = 2        /* the context's learned model predicts the direction        */
};

typedef struct ncg_ctx ncg_ctx;

/* Per-call statistics (host-visible after the call's stream work completes). */
typedef struct ncg_stats {
    uint64_t n_pairs;
    uint64_t n_epa;          /* pairs that went through EPA                   */
    uint64_t n_epa_overflow; /* pairs whose EPA ran in the warp stage          */
    uint64_t gjk_iters;      /* sum over pairs                                */
    uint64_t epa_iters;      /* sum over pairs                                */
    uint32_t kernels_launched;
    uint32_t flags;          /* bit 0: a learned warm-start tensor-core wait
                                timed out (directions fell back to default);
                                bit 1: a hull-stage bulk-copy wait timed out
                                (those pairs read global memory instead) */
    uint64_t n_epa_thread;   /* pairs whose EPA started in the thread stage
                                (the others started in the warp stage)      */
} ncg_stats;

/* ---- context --------------------------------------------------------------- */
/* Creates a context on `device`.  The context owns scratch memory (EPA queue,
 * pair buckets), CUDA graphs and the learned warm-start model. */
int ncg_ctx_create(ncg_ctx** out, int device);
int ncg_ctx_destroy(ncg_ctx* ctx);
int ncg_ctx_set_tolerance(ncg_ctx* ctx, int tolerance);
/* Selects an ncg_arithmetic (no reference counterpart: the reference picks its
 * arithmetic by instantiating N = f32 or f64). */
int ncg_ctx_set_arithmetic(ncg_ctx* ctx, int arithmetic);
int ncg_ctx_set_warm_start(ncg_ctx* ctx, int warm_start);
int ncg_ctx_set_dispatch(ncg_ctx* ctx, int dispatch);
/* Launch tuning (no reference counterpart).  Keys:
 *   NCG_TUNE_HULL_GJK_WARP   0: GJK of ConvexHull pairs one thread per pair
 *                            (default), 1: one warp per pair, v in 2..14: one
 *                            warp per pair for pairs scanning >= 2^v hull points
 *   NCG_TUNE_GJK_BLOCKS      blocks of 128 threads per SM for the thread-per-pair
 *                            GJK kernel; 0 = as many as fit (default)
 *   NCG_TUNE_EPA_BLOCKS      the same for the thread-per-pair EPA kernel
 *   NCG_TUNE_L1_CARVEOUT     shared-memory carveout (percent) preferred by the
 *                            kernels that use no shared memory; -1 = driver
 *                            default, 0 = largest L1 (default)
 *   NCG_TUNE_HULL_STAGE_MIN  warp-per-pair hull GJK: a pair whose ConvexHull
 *                            shapes hold at least this many points has them
 *                            copied into shared memory by the bulk-copy (TMA)
 *                            engine before its first support scan; 0 = never
 *                            (default), at most 2048
 *   NCG_TUNE_HULL_STAGE_CAP  points of that shared-memory stage per warp
 *                            (multiple of 32, 32..2048; default 1024); a hull
 *                            that does not fit is scanned from global memory
 *   NCG_TUNE_HULL_EPA_WARP   v in 2..14: the EPA of ConvexHull pairs scanning
 *                            >= 2^v points whose GJK ran one thread per pair
 *                            starts in the warp stage (warp-parallel support
 *                            scans) instead of the thread stage; 0 = never
 *                            (default: with hulls shared by many pairs the
 *                            thread stage's scans hit L2 and it is faster)
 *   NCG_TUNE_HULL_LOCALITY   1 (default): in a batch whose pairs reference each
 *                            shape four times or more on average, the pairs of
 *                            each ConvexHull size bucket are grouped by the
 *                            index range (1/4096 of the shapes) of their first
 *                            ConvexHull, so that pairs sharing hulls run close
 *                            together and their points stay in L2; 0: not
 * Results do not depend on any of these. */
enum ncg_tune {
    NCG_TUNE_HULL_GJK_WARP = 0,
    NCG_TUNE_GJK_BLOCKS = 1,
    NCG_TUNE_EPA_BLOCKS = 2,
    NCG_TUNE_L1_CARVEOUT = 3,
    NCG_TUNE_HULL_STAGE_MIN = 4,
    NCG_TUNE_HULL_STAGE_CAP = 5,
    NCG_TUNE_HULL_EPA_WARP = 6,
    NCG_TUNE_HULL_LOCALITY = 7
};
#define NCG_N_TUNE 8
int ncg_ctx_set_tuning(ncg_ctx* ctx, int key, int value);

/* Autotuner (no reference counterpart; the reference has no launch tuning).
 * Times `query` (ncg_query_kind; param = prediction or margin) on the given
 * device-resident batch for candidate values of every NCG_TUNE_* key, by
 * coordinate descent from the context's current values (at most two passes;
 * a value is kept when it is at least 1% faster), and leaves the fastest
 * values set in the context.  Each candidate runs once untimed, then `reps`
 * times (1..64) between CUDA events on `stream`; its time is the fastest of
 * those.  The outputs of every candidate are checked against the first
 * candidate's (a digest of every output byte): results must not depend on
 * tuning, and a difference returns NCG_EINTERNAL.  Writes the chosen values
 * (indexed by key, NCG_N_TUNE of them) to out_values and the chosen
 * configuration's time to *out_ms (either may be NULL).  Allocates its own
 * output buffers; synchronises `stream`. */
enum ncg_query_kind {
    NCG_QUERY_CONTACT = 0,
    NCG_QUERY_DISTANCE = 1,
    NCG_QUERY_PROXIMITY = 2,
    NCG_QUERY_CLOSEST_POINTS = 3
};
int ncg_autotune(ncg_ctx* ctx, const ncg_batch* batch, int query, float param, int reps, int* out_values,
                 float* out_ms, void* stream);
int ncg_ctx_get_tuning(ncg_ctx* ctx, int key, int* value);
int ncg_sync(ncg_ctx* ctx, void* stream);
int ncg_get_stats(ncg_ctx* ctx, ncg_stats* out);

/* Stage timing: when enabled, each batch call records CUDA events between its
 * kernel launches on the caller's stream.  ncg_get_stage_ms fills up to
 * n_max durations in milliseconds (order: classify, gjk_thread, gjk_warp,
 * epa_thread, epa_warp, epa_wide) of the last call and returns
 * how many it wrote; it synchronises on the last call's events.  No reference
 * counterpart (the reference has no instrumentation). */
#define NCG_N_STAGES 6
int ncg_ctx_set_profiling(ncg_ctx* ctx, int enabled);
int ncg_get_stage_ms(ncg_ctx* ctx, float* ms, int n_max);
const char* ncg_last_error(void);
int ncg_abi_version(void);

/* ---- batched queries on device memory (asynchronous) ----------------------- */

/* contact_support_map_support_map_with_params for every pair.
 * out[i] is valid when has_contact[i] == 1.  out_dir (nullable, 3 floats per
 * pair) receives the direction the reference returns for reuse as the next
 * init_dir.  iters (nullable) = gjk_iterations | (epa_iterations << 16). */
int ncg_contact_batch(ncg_ctx* ctx, const ncg_batch* batch, float prediction,
                      ncg_contact* out, uint8_t* has_contact, float* out_dir,
                      uint32_t* status, uint32_t* iters, void* stream);

/* ---- learned warm start (no reference counterpart) --------------------------
 * A 39 -> 128 -> 128 -> 4 MLP (GELU) predicts GJK's first search direction
 * and the sign of the separation from the relative pose and two 16-float
 * shape descriptors.  Parameters: NCG_MLP_N_PARAMS f32 values laid out
 * W1[128][48], b1[128], W2[128][128], b2[128], W3[4][128], b3[4] (inputs
 * 39..47 are zero padding).  With NCG_WARM_MLP the context runs the network
 * (tcgen05 tensor cores, bf16 operands, f32 accumulation) before GJK and uses
 * its unit direction as init_dir of every query (contact, distance, proximity,
 * closest points); GJK and EPA still run to their own termination.  Measured:
 * contact with prediction 0 stops at the first separating axis and its GJK
 * iterations hardly change; closest points gain only from the exact final
 * direction, and an approximate one (the network's) costs a few percent more
 * iterations than the reference's default start.   Training entry points work on device buffers:
 *   ncg_mlp_features   shape descriptors (desc: 16 floats per shape) and the
 *                      48 input features of every pair (X: 48 floats per pair)
 *   ncg_mlp_infer      the network's world-space unit direction per pair
 *   ncg_mlp_grad       mean-loss gradient of a batch of n samples: X [n][48],
 *                      labels [n][4] = unit direction in the first shape's
 *                      frame, then 1 (intersecting) or 0; loss = (1 - cos) +
 *                      logit_weight * BCE.  partial needs ceil(n/128) *
 *                      (NCG_MLP_N_PARAMS + 4) floats; grad receives
 *                      NCG_MLP_N_PARAMS gradients then the loss, the
 *                      direction loss and the logit loss
 *   ncg_mlp_adam       one Adam step (step counts from 1)
 * err (device uint32) gets bit 0 when a tensor-core wait times out. */
#define NCG_MLP_N_INPUTS 48
#define NCG_MLP_N_PARAMS 23300
int ncg_mlp_n_params(void);
int ncg_ctx_set_mlp_params(ncg_ctx* ctx, const float* params, int n);
int ncg_mlp_features(const ncg_batch* batch, float* desc, float* X, void* stream);
int ncg_mlp_infer(const ncg_batch* batch, const float* params, float* desc, float* init_dir, uint32_t* err,
                  void* stream);
int ncg_mlp_grad(const float* params, const float* X, const float* labels, uint64_t n, float logit_weight,
                 float* partial, float* grad, uint32_t* err, void* stream);
int ncg_mlp_adam(float* params, float* m, float* v, const float* grad, float lr, float beta1, float beta2,
                 float eps, int step, void* stream);

/* ---- CUDA graphs of one query (no reference counterpart) ------------------
 * ncg_contact_graph_create captures one ncg_contact_batch call with these
 * arguments into a CUDA graph owned by the context.  Each ncg_graph_launch
 * re-runs the query on whatever the batch's device buffers hold when the
 * replay executes (poses updated in place between frames, an init_dir buffer
 * refreshed from out_dir), with the context's tolerance, dispatch and warm
 * start as they were at capture time.  out_dir may alias batch->init_dir: each
 * pair reads its init_dir before its out_dir is written, which gives the
 * previous-frame direction reuse of the reference's manifold generator
 * (convex_polyhedron_convex_polyhedron_manifold_generator.rs:96-145).
 * Replays and other calls on the same context share its scratch: serialise
 * them on one stream.  The graph is destroyed with ncg_graph_destroy or with
 * the context. */
typedef struct ncg_graph ncg_graph;
int ncg_contact_graph_create(ncg_ctx* ctx, const ncg_batch* batch, float prediction,
                             ncg_contact* out, uint8_t* has_contact, float* out_dir,
                             uint32_t* status, uint32_t* iters, ncg_graph** graph);
int ncg_graph_launch(ncg_graph* graph, void* stream);
int ncg_graph_destroy(ncg_graph* graph);

/* distance_support_map_support_map_with_params for every pair. */
int ncg_distance_batch(ncg_ctx* ctx, const ncg_batch* batch, float* out_dist,
                       uint32_t* status, uint32_t* iters, void* stream);

/* proximity_support_map_support_map_with_params for every pair.  Returns
 * NCG_EINVAL when margin < 0 (the reference asserts). out_sep_axis nullable. */
int ncg_proximity_batch(ncg_ctx* ctx, const ncg_batch* batch, float margin,
                        uint8_t* out_prox, float* out_sep_axis, uint32_t* status,
                        uint32_t* iters, void* stream);

/* closest_points_support_map_support_map_with_params for every pair.
 * out_points: 6 floats per pair (p1, p2), valid when tag == NCG_CP_WITHIN_MARGIN. */
int ncg_closest_points_batch(ncg_ctx* ctx, const ncg_batch* batch, float prediction,
                             uint8_t* out_tag, float* out_points, uint32_t* status,
                             uint32_t* iters, void* stream);

/* query::time_of_impact for every pair (time_of_impact.rs:63-90 over
 * time_of_impact_support_map_support_map.rs:10-127; Ball-Ball pairs take
 * time_of_impact_ball_ball.rs:9-62 under NCG_DISPATCH_QUERY).  vel1, vel2:
 * 3 floats per pair (linear velocities).  max_toi >= FLT_MAX (or +inf) means
 * unbounded.  Returns NCG_EINVAL when max_toi or target_distance is negative
 * or NaN.  has_toi[i] = 1 for Some; out[i] is then the TOI.  iters nullable:
 * ray-cast iterations plus, for a dilated toi of zero, the GJK iterations of
 * the closest-points refinement. */
int ncg_time_of_impact_batch(ncg_ctx* ctx, const ncg_batch* batch, const float* vel1,
                             const float* vel2, float max_toi, float target_distance,
                             ncg_toi* out, uint8_t* has_toi, uint32_t* status,
                             uint32_t* iters, void* stream);

/* RayCast::toi_and_normal_with_ray of support-map shapes for every ray
 * (src/query/ray/ray_support_map.rs:14-56 and its RayCast impls :58-110,
 * gjk::cast_ray src/query/algorithms/gjk.rs:180-194): ray i against
 * shapes[g1[i]] at pose m1[i] (m2, g2 and init_dir unused).  rays: origin[3],
 * dir[3] per ray, world frame; the toi is in units of |dir|.  Every shape kind
 * takes the GJK ray cast (the reference's Ball and Cuboid have analytic
 * RayCast impls of their own).  solid = 0: a ray starting inside returns its
 * exit.  out_normal nullable (3 floats per ray, world frame).  Returns
 * NCG_EINVAL when max_toi is negative or NaN. */
int ncg_ray_cast_batch(ncg_ctx* ctx, const ncg_batch* batch, const float* rays, float max_toi,
                       int solid, float* out_toi, float* out_normal, uint8_t* has_hit,
                       uint32_t* status, uint32_t* iters, void* stream);

/* ConvexPolyhedronConvexPolyhedronManifoldGenerator::generate_contacts
 * (src/pipeline/narrow_phase/contact_generator/convex_polyhedron_convex_polyhedron_manifold_generator.rs:84-176)
 * for every pair: contact_support_map_support_map_with_params with
 * prediction.linear (init_dir = last_gjk_dir under NCG_WARM_INIT_DIR), then for
 * Cuboid pairs the support faces (depth > 0) or the support features within
 * the angular tolerances (cuboid.rs:279-405), their clipping
 * (convex_polygonal_feature3.rs:217-339) and the contacts handed to the
 * manifold (add_contact_to_manifold's feature checks; the manifold's
 * persistence cache is the caller's).  contact / has_contact / out_dir receive
 * the contact query's results (out_dir may alias batch->init_dir: the next
 * frame's last_gjk_dir).  Pairs that are not two Cuboids get their single
 * contact with NCG_STATUS_NOT_POLYHEDRA. */
int ncg_manifold_batch(ncg_ctx* ctx, const ncg_batch* batch, float prediction, float angular1,
                       float angular2, ncg_contact* contact, uint8_t* has_contact, float* out_dir,
                       ncg_manifold* out, uint32_t* status, void* stream);

/* ---- ConvexHull face topology ----------------------------------------------
 * The polyhedral structure of every ConvexHull shape of a shape table, as
 * ConvexHull::try_new (src/shape/convex.rs:88-328) builds it from the hull's
 * points and the triangles of their convex hull: polygonal faces (triangles
 * whose normals differ by less than sqrt(f32::EPSILON) merged), edges with
 * their unit directions, and the faces and edges around each vertex.  Ids are
 * local to the hull (point i of a hull is vertex i: the points are not
 * reordered; this is try_new on the hull's own points, not try_from_points,
 * whose hull step renormalises and reorders them).  ncg_hull_topology_build
 * fills `out` with host arrays it allocates (free them with
 * ncg_hull_topology_release); n_failed counts hulls left without a topology
 * (degenerate points, or a check of try_new failed).  For
 * ncg_manifold_batch_hulls, copy the arrays to the device and pass a struct of
 * device pointers with the same counts.  Shape set-up, not part of a query. */
typedef struct ncg_hull_topology {
    uint64_t n_shapes, n_hull_points, n_faces, n_face_slots, n_edges, n_vertex_slots;
    const uint32_t* shape;         /* [n_shapes][4]: first face, face count, first edge, edge count */
    const float* face_normal;      /* [n_faces][4]: unit outward normal, 0 */
    const uint32_t* face_range;    /* [n_faces][2]: first slot in face_vertex / face_edge, count */
    const uint32_t* face_vertex;   /* [n_face_slots]: hull-local point id, counter-clockwise */
    const uint32_t* face_edge;     /* [n_face_slots]: hull-local id of the edge to the next vertex */
    const uint32_t* edge_vertex;   /* [n_edges][2]: hull-local point ids */
    const float* edge_dir;         /* [n_edges][4]: unit direction, 0 */
    const uint32_t* vertex_range;  /* [n_hull_points][2]: first slot in vertex_face / vertex_edge, count */
    const uint32_t* vertex_face;   /* [n_vertex_slots]: hull-local face id */
    const uint32_t* vertex_edge;   /* [n_vertex_slots]: hull-local edge id */
} ncg_hull_topology;
int ncg_hull_topology_build(const ncg_shape* shapes, uint32_t n_shapes, const float* hull_points,
                            uint64_t n_hull_points, ncg_hull_topology* out, uint32_t* n_failed);
int ncg_hull_topology_release(ncg_hull_topology* topology);
/* ncg_manifold_batch with ConvexHull shapes as polyhedra (ConvexHull's
 * ConvexPolyhedron impl, convex.rs:425-546: support_face_toward takes the face
 * whose normal has the largest dot product with the direction,
 * support_feature_toward the support point's adjacent face or edge within the
 * angular tolerance, else the vertex) for every pair of Cuboid and ConvexHull
 * shapes; `topology` holds device pointers (NULL: as ncg_manifold_batch).  A
 * ConvexHull face of more than NCG_POLY_MAX vertices, or a hull without a
 * topology, gives the pair its single contact with NCG_STATUS_NOT_POLYHEDRA. */
#define NCG_POLY_MAX 32
int ncg_manifold_batch_hulls(ncg_ctx* ctx, const ncg_batch* batch, const ncg_hull_topology* topology,
                             float prediction, float angular1, float angular2, ncg_contact* contact,
                             uint8_t* has_contact, float* out_dir, ncg_manifold* out, uint32_t* status,
                             void* stream);

/* ---- bounding volumes and the broad phase ----------------------------------
 * ncg_aabb_batch: HasBoundingVolume<AABB>::bounding_volume of shapes[g1[i]] at
 * m1[i] for every entry (src/bounding_volume/aabb_ball.rs, aabb_cuboid.rs,
 * aabb_support_map.rs, aabb_convex.rs, aabb_utils.rs:8-74); out_aabbs: mins[3],
 * maxs[3] per entry (device); a bad shape gets NaN bounds and
 * NCG_STATUS_BAD_INPUT.  m2, g2, init_dir unused.
 *
 * ncg_broad_phase: DBVTBroadPhase (src/pipeline/broad_phase/dbvt_broad_phase.rs)
 * over proxies 0 .. n-1.  ncg_bp_update(boxes) = deferred_set_bounding_volume
 * for every proxy (:322-347: a stored box that does not contain the new one is
 * replaced by new.loosened(margin)) followed by update (:174-258).  The pair
 * set is every intersecting pair of stored boxes; started / stopped are the
 * pairs that entered / left it (interference_started / _stopped).  Pairs are
 * (lower id, higher id) uint32 pairs sorted lexicographically, in device
 * memory owned by the broad phase and valid until its next update.  The proxy
 * count may grow between updates, not shrink: a proxy with a NaN bound has no
 * pairs (remove).  Every pair is allowed (no is_interference_allowed filter).
 * ncg_bp_update synchronises the stream. */
typedef struct ncg_broad_phase ncg_broad_phase;
int ncg_aabb_batch(ncg_ctx* ctx, const ncg_batch* batch, float* out_aabbs, uint32_t* status,
                   void* stream);
int ncg_bp_create(ncg_ctx* ctx, float margin, ncg_broad_phase** out);
int ncg_bp_update(ncg_broad_phase* bp, const float* aabbs, uint32_t n_proxies, void* stream);
int ncg_bp_results(ncg_broad_phase* bp, uint64_t* n_pairs, uint64_t* n_started, uint64_t* n_stopped,
                   const uint32_t** pairs, const uint32_t** started, const uint32_t** stopped);
/* Copies the last update's pairs / started / stopped (2 uint32 each) into
 * caller buffers (device or host; NULL skips one), asynchronously on stream. */
int ncg_bp_copy(ncg_broad_phase* bp, uint32_t* pairs, uint32_t* started, uint32_t* stopped, void* stream);
int ncg_bp_destroy(ncg_broad_phase* bp);
/* The narrow-phase batch of a pair list (device): m1/g1 and m2/g2 of pair k are
 * the pose and shape id of proxies pairs[2k] and pairs[2k+1] (the collision
 * world's step from the broad phase's pairs to the narrow phase). */
int ncg_gather_pairs(ncg_ctx* ctx, const ncg_pose* poses, const uint32_t* shape_ids, const uint32_t* pairs,
                     uint64_t n_pairs, ncg_pose* m1, uint32_t* g1, ncg_pose* m2, uint32_t* g2, void* stream);

/* ---- the same on host memory (synchronous; copies in and out) -------------- */
int ncg_contact_batch_host(ncg_ctx* ctx, const ncg_batch* batch, float prediction,
                           ncg_contact* out, uint8_t* has_contact, float* out_dir,
                           uint32_t* status);
int ncg_distance_batch_host(ncg_ctx* ctx, const ncg_batch* batch, float* out_dist,
                            uint32_t* status);
int ncg_proximity_batch_host(ncg_ctx* ctx, const ncg_batch* batch, float margin,
                             uint8_t* out_prox, float* out_sep_axis, uint32_t* status);

/* ---- contact without any device allocation --------------------------------
 * For callers that cannot allocate device memory at the moment they need
 * contacts: code recording a CUDA graph through stream capture without a graph
 * memory pool, real-time simulation loops whose allocator is frozen after
 * start-up, and host runtimes (game engines, FFI hosts) that own every device
 * allocation themselves.  This entry point needs no ncg_ctx and never calls
 * cudaMalloc, cudaFree or any allocating routine: its scratch (pair lists, EPA
 * work items and one global-memory EPA slab) is a fixed array of
 * NCG_NOALLOC_SCRATCH_BYTES (8.0 MiB) compiled into the library,
 * which every GPU that loads the library holds until the process exits.
 * Limit: at most NCG_NOALLOC_MAX_PAIRS pairs per call; a larger batch returns
 * NCG_EINVAL with a message in ncg_last_error().
 * The first call on a device performs a one-time set-up with that device
 * current (it looks up the array's device address and the launch limits):
 * make that first call before any stream capture.  Every call on a device
 * shares the one array and the array keeps the previous call's contents (the
 * call clears what must start at zero), so calls that overlap on the GPU —
 * different streams, or concurrent host threads — race and corrupt each
 * other's results: serialise them.
 * `stream` must belong to the current device (checked: NCG_EINVAL otherwise).
 * `tolerance` is an ncg_tolerance; batch->init_dir, when not NULL, is the
 * first GJK direction of every pair.  Every pair runs
 * contact_support_map_support_map (NCG_DISPATCH_SUPPORT_MAP): results equal
 * those of ncg_contact_batch on a context with that dispatch (the default),
 * the same tolerance set and, when init_dir is given, NCG_WARM_INIT_DIR; a
 * context using NCG_DISPATCH_QUERY routes Ball pairs differently.
 * EPA runs in three stores: 128 vertices, then 1280 (both in shared memory),
 * then the array's one 10240-vertex slab, which a single warp drains: pairs
 * whose polytope outgrows 1280 vertices (deep, nearly concentric curved
 * pairs) run one after another there, which bounds a call's latency from
 * below by their summed EPA time.
 * This entry point has no counterpart in the reference. */
#define NCG_NOALLOC_MAX_PAIRS 32768
#define NCG_NOALLOC_SCRATCH_BYTES 8420608
int ncg_contact_batch_noalloc(const ncg_batch* batch, float prediction, int tolerance,
                              ncg_contact* out, uint8_t* has_contact, float* out_dir,
                              uint32_t* status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* NCG_H */
