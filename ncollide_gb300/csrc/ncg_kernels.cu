// ncg_kernels.cu — the EPA stages of a batched contact query, the host side
// of every query and the C ABI of include/ncg.h.
//
// One batch call runs, on one stream and without host synchronisation:
//   1. classify, bucket   (ncg_gjk.cu) 1 thread/pair: validates the pair and
//                         counting-sorts it by cost bucket (shape kinds, hull
//                         sizes).
//   2. gjk_thread         (ncg_gjk.cu) 1 thread/pair over the analytic list,
//                         then over the ConvexHull list (or 1 warp/pair over
//                         the ConvexHull list with NCG_TUNE_HULL_GJK_WARP).
//   3. epa_thread         contact only, intersecting pairs: 1 thread/pair,
//                         polytope of up to 64 vertices in local memory.
//   4. epa warp stage     pairs that outgrew the thread stage: 1 warp/pair,
//                         up to 1280 vertices in a global-memory slab per
//                         warp, 12 warps per SM; pairs of two curved shapes
//                         (the longest polytopes) first.
//   5. epa wide stage     pairs that outgrew the warp stage: up to 10240
//                         vertices, one slab per SM.
// A pair that outgrows a stage is re-run by the next one from GJK's simplex.
// Pairs are independent; the GJK stage writes its outputs directly or appends
// the final simplex to the EPA queue.  The no-allocation entry point runs the
// same GJK stage, then EPA with 128 and 1280 vertices in shared memory and a
// static global slab.

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ncg.h"
#include "ncg_core.cuh"
#include "ncg_mlp.h"
#include "ncg_toi.h"
#include "ncg_bp.h"
#include "ncg_manifold.h"
#include "ncg_epa.cuh"
#include "ncg_query.cuh"
#include "ncg_pipeline.cuh"
#include "ncg_sort.cuh"

using namespace ncg;

namespace {

thread_local std::string g_last_error;

// ------------------------------------------------------------------ host side
}  // namespace
namespace ncg {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace ncg
namespace {

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

// Tolerance constants in f64, split into double-words.
// REFERENCE: the reference's own f32 constants (eps = f32::EPSILON).
// PRECISE: the tests that classify (origin on the simplex, origin inside the
// tetrahedron, EPA face checks and visibility) keep f32::EPSILON, the noise
// floor of f32 support points; the tests that decide how far GJK refines
// (add_point's degeneracy threshold, the relative gap sqrt(10 eps)) use
// f64::EPSILON as the reference built with f64; EPA terminates at 1e-6
// absolute (the f64 reference's 100 eps is below f32 support noise).
Tol make_tol(int mode) {
    Tol t;
    double e = (double)FLT_EPSILON;
    t.eps = dw_split(e);
    t.eps_tol = dw_split(e * 10.0);
    t.eps_rel = dw_split(std::sqrt(e * 10.0));
    t.epa_eps_tol = dw_split(e * 100.0);
    double a = e * 100.0;
    t.affine_eps = dw_split(a * a);
    t.add_tol = t.eps_tol;
    if (mode == NCG_TOL_PRECISE) {
        t.eps_rel = dw_split(std::sqrt(10.0 * (double)DBL_EPSILON));
        t.add_tol = dw_split(10.0 * (double)DBL_EPSILON);
        t.epa_eps_tol = dw_split(1e-6);
    }
    t.best_on_failure = mode == NCG_TOL_PRECISE ? 1 : 0;
    t.eps_tol_f = t.eps_tol.h;
    t.affine_eps_f = t.affine_eps.h;
    t.init_eps = FLT_EPSILON;
    return t;
}

// The same sets for the f32 build, each constant computed in f32 as the
// reference's f32 path computes it (eps_tol = 10 eps, eps_rel = sqrt(eps_tol),
// 100 eps, (100 eps)^2); the PRECISE set's f64 constants rounded to f32.
Tol make_tol_f32(int mode) {
    Tol t;
    const float e = FLT_EPSILON;
    const float et = e * 10.0f, e100 = e * 100.0f;
    auto f = [](float x) { return dw_host{x, 0.0f}; };
    t.eps = f(e);
    t.eps_tol = f(et);
    t.eps_rel = f(sqrtf(et));
    t.epa_eps_tol = f(e100);
    t.affine_eps = f(e100 * e100);
    t.add_tol = t.eps_tol;
    if (mode == NCG_TOL_PRECISE) {
        t.eps_rel = f((float)std::sqrt(10.0 * (double)DBL_EPSILON));
        t.add_tol = f((float)(10.0 * (double)DBL_EPSILON));
        t.epa_eps_tol = f((float)1e-6);
    }
    t.best_on_failure = mode == NCG_TOL_PRECISE ? 1 : 0;
    t.eps_tol_f = t.eps_tol.h;
    t.affine_eps_f = t.affine_eps.h;
    t.init_eps = FLT_EPSILON;
    return t;
}

// The launchers of one build of the GJK and EPA stages.
struct Stages {
    decltype(&dwa::gjk_launch_sort) sort;
    decltype(&dwa::gjk_launch_thread) gjk_thread;
    decltype(&dwa::gjk_launch_warp) gjk_warp;
    decltype(&dwa::epa_launch_thread) epa_thread;
    decltype(&dwa::epa_launch_warp) epa_warp;
};
const Stages STAGES_SPLIT{dwa::gjk_launch_sort, dwa::gjk_launch_thread, dwa::gjk_launch_warp, dwa::epa_launch_thread,
                          dwa::epa_launch_warp};
const Stages STAGES_F32{f32a::gjk_launch_sort, f32a::gjk_launch_thread, f32a::gjk_launch_warp,
                        f32a::epa_launch_thread, f32a::epa_launch_warp};

}  // namespace

// Stage-timing events of one call: a start mark and one per launch group.
constexpr int NCG_N_MARKS = NCG_N_STAGES + 2;

struct ncg_ctx {
    int device = 0;
    int num_sms = 0;
    int tol_mode = NCG_TOL_REFERENCE;
    int arith = NCG_ARITH_SPLIT;
    int warm = NCG_WARM_NONE;
    int dispatch = NCG_DISPATCH_SUPPORT_MAP;
    int hull_gjk_warp = 0;  // GJK of ConvexHull pairs: 0 one thread per pair, 1 one warp per pair
    int hull_epa_warp = 0;  // v >= 2: EPA of ConvexHull pairs scanning >= 2^v points starts in the warp stage
    int hull_locality = 1;  // 1: ConvexHull pairs sorted by hull index range when the batch reuses its shapes
    int occ_thread = 1, occ_warp = 1, occ_ethread = 1;
    int occ_smem[2] = {1, 1};  // warps per SM of k_epa with a store of EpaTier<1> / <2> in shared memory
    int occ_global = 1;        // warps per SM of k_epa on global slabs
    int gjk_blocks = 0, epa_blocks = 0, l1_carveout = 0;
    // warp-per-pair hull GJK: stage the pair's hull points in shared memory
    // when they number at least hstage_min (0: never), hstage_cap points per warp
    int hstage_min = 0, hstage_cap = 1024, occ_hstage = 0;
    char* scratch = nullptr;
    size_t scratch_cap_pairs = 0;
    char* slabs = nullptr;  // warp-stage slabs, then wide-stage slabs
    int n_slabs[2] = {0, 0};
    size_t slab_bytes[2] = {0, 0};
    DevCounters* host_ctr = nullptr;  // pinned
    ncg_stats last{};
    uint32_t launches = 0;
    // host-API staging buffers
    char* stage = nullptr;
    size_t stage_cap = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host entry points: the hull-point copy
    cudaEvent_t hull_ready = nullptr;    // recorded on copy_stream after that copy
    int profiling = 0;
    std::vector<ncg_graph*> graphs;  // destroyed with the context
    float* mlp_params = nullptr;     // NCG_MLP_N_PARAMS floats (device)
    bool mlp_ready = false;          // kernel attributes set on this device
    float* desc_buf = nullptr;       // shape descriptors for the network
    size_t desc_cap = 0;
    float* idir_buf = nullptr;       // the network's init_dir per pair
    size_t idir_cap = 0;
    uint32_t graph_launches = 0;     // kernels in a captured query
    int n_marks = 0;
    int mark_stage[NCG_N_MARKS];
    cudaEvent_t marks[NCG_N_MARKS] = {};
};

namespace {

// Spill records of the thread stage: one per 32 pairs of capacity (the
// thread stage's overflow is ~1-3% of the pairs on mixed workloads; beyond
// the records, pairs restart from GJK's simplex as without them).
uint64_t spill_records(uint64_t cap) { return cap / 32 < 256 ? 256 : cap / 32; }

bool ensure_scratch(ncg_ctx* c, uint64_t n) {
    if (n <= c->scratch_cap_pairs && c->scratch) return true;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    uint64_t cap = n < 1024 ? 1024 : n;
    size_t bytes = (2 + N_EPA_QUEUES) * 4 * cap + sizeof(EpaItem) * cap + CTR_SLOT + 1024 + 4 * cap +
                   SPILL_BYTES * spill_records(cap) + 256;
    if (!cuda_ok(cudaMalloc(&c->scratch, bytes), "cudaMalloc(scratch)")) return false;
    c->scratch_cap_pairs = cap;
    return true;
}

// Buffers of the learned warm start (shape descriptors, one init_dir per pair).
int ensure_mlp_buffers(ncg_ctx* c, const ncg_batch* b) {
    if (!c->mlp_params) { g_last_error = "NCG_WARM_MLP without parameters (ncg_ctx_set_mlp_params)"; return NCG_EINVAL; }
    if (!c->mlp_ready) {
        if (mlp_prepare() != NCG_OK) return NCG_ECUDA;
        c->mlp_ready = true;
    }
    if (c->desc_cap < b->n_shapes) {
        if (c->desc_buf) cudaFree(c->desc_buf);
        c->desc_buf = nullptr;
        c->desc_cap = 0;
        const size_t cap = b->n_shapes < 1024 ? 1024 : b->n_shapes;
        if (!cuda_ok(cudaMalloc(&c->desc_buf, 64 * cap), "cudaMalloc(desc)")) return NCG_ENOMEM;
        c->desc_cap = cap;
    }
    if (c->idir_cap < b->n_pairs) {
        if (c->idir_buf) cudaFree(c->idir_buf);
        c->idir_buf = nullptr;
        c->idir_cap = 0;
        if (!cuda_ok(cudaMalloc(&c->idir_buf, 12 * (size_t)b->n_pairs), "cudaMalloc(init_dir)")) return NCG_ENOMEM;
        c->idir_cap = b->n_pairs;
    }
    return NCG_OK;
}

Scratch carve_scratch(ncg_ctx* c) {
    Scratch s;
    uint64_t cap = c->scratch_cap_pairs;
    char* p = c->scratch;
    s.ctr = (DevCounters*)p; p += CTR_SLOT;
    s.items = (EpaItem*)p; p += sizeof(EpaItem) * cap;
    s.bucket = (uint8_t*)p; p += 4 * cap;
    s.sub = (uint16_t*)(s.bucket + 2 * cap);  // the bucket array's region holds 4 bytes per pair
    s.loc_shift = 32;
    s.sorted = (uint32_t*)p; p += 4 * cap;
    for (int q = 0; q < N_EPA_QUEUES; ++q) { s.queue[q] = (uint32_t*)p; p += 4 * cap; }
    s.spill_of = (uint32_t*)p; p += 4 * cap;
    p = (char*)(((uintptr_t)p + 255) & ~uintptr_t(255));
    s.spill = p;
    s.spill_bytes = SPILL_BYTES;
    s.spill_cap = (uint32_t)spill_records(cap);
    s.slabs[0] = c->slabs;
    s.slabs[1] = c->slabs + c->slab_bytes[0] * c->n_slabs[0];
    for (int t = 0; t < 2; ++t) {
        s.slab_bytes[t] = c->slab_bytes[t];
        s.n_slabs[t] = c->n_slabs[t];
    }
    return s;
}

// Resident blocks per SM of every kernel (and the shared-memory limit of k_epa).
struct Limits {
    int occ_thread = 1, occ_warp = 1, occ_ethread = 1, occ_global = 1;
    int occ_smem[2] = {1, 1};
};
Limits launch_limits() {
    Limits l;
    // grids are sized from the double-word build's kernels (the f32 build's
    // use no more registers)
    dwa::gjk_occupancy(&l.occ_thread, &l.occ_warp);
    dwa::epa_occupancy(&l.occ_ethread, &l.occ_global, l.occ_smem);
    int* all[] = {&l.occ_thread, &l.occ_warp, &l.occ_ethread, &l.occ_global, &l.occ_smem[0], &l.occ_smem[1]};
    for (int* v : all)
        if (*v < 1) *v = 1;
    if (l.occ_global > WARP_STAGE_MAX_PER_SM) l.occ_global = WARP_STAGE_MAX_PER_SM;
    return l;
}

// Shared-memory carveout preference of the kernels without shared memory
// (their local-memory and hull traffic wants the largest L1).
bool set_carveout(int pct) {
    bool ok = true;
    ok &= cuda_ok(dwa::gjk_set_carveout(pct), "carveout(k_gjk_thread)");
    ok &= cuda_ok(dwa::epa_set_carveout(pct), "carveout(k_epa_thread)");
    ok &= cuda_ok(f32a::gjk_set_carveout(pct), "carveout(k_gjk_thread, f32)");
    ok &= cuda_ok(f32a::epa_set_carveout(pct), "carveout(k_epa_thread, f32)");
    return ok;
}

// Runs one batched query on stream st.  When `hull_ready` is given (the host
// entry points), the hull points are still being copied on another stream:
// the analytic pairs' GJK and, for contact, their thread-stage EPA (queue 0)
// need none of them and overlap the copy; the stream waits for the event
// before the first kernel that reads hull points, and the ConvexHull pairs'
// thread-stage EPA runs after their GJK (queue 4).
int run_query(ncg_ctx* c, const ncg_batch* b, int query, float param, const Outputs& o, cudaStream_t st,
              cudaEvent_t hull_ready = nullptr) {
    if (!c || !b) { g_last_error = "null context or batch"; return NCG_EINVAL; }
    if (b->n_pairs == 0) return NCG_OK;
    if (b->n_pairs > 0xffffffffull) { g_last_error = "more than 2^32-1 pairs"; return NCG_EINVAL; }
    if (!b->shapes || !b->m1 || !b->m2 || !b->g1 || !b->g2 || !o.status) {
        g_last_error = "null required pointer";
        return NCG_EINVAL;
    }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    if (!ensure_scratch(c, b->n_pairs)) return NCG_ENOMEM;
    Scratch s = carve_scratch(c);
    if (c->hull_locality && b->n_shapes > 0 && b->n_pairs >= 2 * (uint64_t)b->n_shapes) {
        // a batch whose pairs reference each shape four times or more on
        // average: HULL_SUB sub-buckets of consecutive shape indices
        uint32_t shift = 0;
        while (shift < 31 && ((b->n_shapes - 1) >> shift) >= (uint64_t)HULL_SUB) ++shift;
        s.loc_shift = shift;
    }
    QueryParams qp;
    qp.query = query;
    qp.dispatch = c->dispatch;
    qp.use_init_dir = (c->warm == NCG_WARM_INIT_DIR && b->init_dir) ? 1 : 0;
    qp.gjk_max_iter = 10000;
    qp.epa_max_iter = 10000;
    const bool f32 = c->arith == NCG_ARITH_F32;
    const Stages& sg = f32 ? STAGES_F32 : STAGES_SPLIT;
    qp.param = f32 ? dw_host{param, 0.0f} : dw_split((double)param);
    qp.tol = f32 ? make_tol_f32(c->tol_mode) : make_tol(c->tol_mode);
    ncg_batch bb = *b;
    uint32_t launches = 0;
    c->n_marks = 0;
    auto mark = [&](int stage) {
        if (!c->profiling) return;
        c->mark_stage[c->n_marks] = stage;
        cudaEventRecord(c->marks[c->n_marks++], st);
    };
    if (!cuda_ok(cudaMemsetAsync(s.ctr, 0, sizeof(DevCounters), st), "memset counters")) return NCG_ECUDA;
    if (c->warm == NCG_WARM_MLP) {
        // the network's start direction replaces the default one (contact and
        // proximity start from normalize(t2 - t1) in the reference, distance
        // and closest points from t1 - t2; the *_with_params wrappers take it
        // as init_dir); the shape descriptors read hull points
        if (hull_ready && !cuda_ok(cudaStreamWaitEvent(st, hull_ready, 0), "cudaStreamWaitEvent")) return NCG_ECUDA;
        int rc = ensure_mlp_buffers(c, b);
        if (rc != NCG_OK) return rc;
        rc = mlp_shape_desc(bb, c->desc_buf, st);
        if (rc == NCG_OK) rc = mlp_infer(bb, c->mlp_params, c->desc_buf, c->idir_buf, &s.ctr->mlp_err, c->num_sms, st);
        if (rc != NCG_OK) return rc;
        bb.init_dir = c->idir_buf;
        qp.use_init_dir = 1;
        launches += 2;
    }
    mark(-1);
    sg.sort(bb, qp, o, s, st);
    mark(0);
    const int gjk_grid = c->num_sms * (c->gjk_blocks > 0 ? c->gjk_blocks : c->occ_thread);
    const int epa_grid = c->num_sms * (c->epa_blocks > 0 ? c->epa_blocks : c->occ_ethread);
    sg.gjk_thread(gjk_grid, bb, qp, o, s, 0, 0, 0, 0, st);
    mark(1);
    launches += 4;
    // With the hull points still in flight, the analytic pairs' thread-stage
    // EPA runs first (it reads no hull points); otherwise one thread-stage
    // launch serves both lists (a second launch adds a tail of ~1 ms).
    const bool split = query == Q_CONTACT && hull_ready != nullptr;
    const int hull_queue = split ? Q_THREAD_HULL : 0;
    if (split) {
        sg.epa_thread(epa_grid, bb, qp, o, s, 0, st);
        mark(3);
        launches += 1;
    }
    if (hull_ready && !cuda_ok(cudaStreamWaitEvent(st, hull_ready, 0), "cudaStreamWaitEvent")) return NCG_ECUDA;
    // hull pairs of the first warp_buckets buckets (largest hulls) one warp per pair
    const int warp_buckets = c->hull_gjk_warp == 0   ? 0
                             : c->hull_gjk_warp == 1 ? NB_HULL
                                                     : std::max(0, std::min(NB_HULL, 3 + NB_HULL - c->hull_gjk_warp));
    if (warp_buckets > 0) {
        const bool staged = c->hstage_min > 0 && c->occ_hstage > 0;
        sg.gjk_warp(c->num_sms * (staged ? c->occ_hstage : c->occ_warp), bb, qp, o, s, warp_buckets,
                    staged ? (uint32_t)c->hstage_min : 0u, (uint32_t)c->hstage_cap, st);
    }
    const int epa_warp_buckets =
        c->hull_epa_warp < 2 ? 0 : std::max(0, std::min(NB_HULL, 3 + NB_HULL - c->hull_epa_warp));
    if (warp_buckets < NB_HULL)
        sg.gjk_thread(gjk_grid, bb, qp, o, s, 1, warp_buckets, hull_queue, query == Q_CONTACT ? epa_warp_buckets : 0,
                      st);
    mark(2);
    launches += (warp_buckets > 0 ? 1 : 0) + (warp_buckets < NB_HULL ? 1 : 0);
    if (query == Q_CONTACT) {
        sg.epa_thread(epa_grid, bb, qp, o, s, hull_queue, st);
        mark(3);
        // warp stage: the thread stage's overflow, pairs of curved shapes first
        sg.epa_warp(c->n_slabs[0], 0, bb, qp, o, s, caps<2>(Q_WARP_LONG, Q_WARP, 3, 0), st);
        mark(4);
        sg.epa_warp(c->n_slabs[1], 0, bb, qp, o, s, caps<3>(3, -1, -1, 1), st);
        mark(5);
        launches += 3;
    }
    if (!cuda_ok(cudaGetLastError(), "kernel launch")) return NCG_ECUDA;
    if (!cuda_ok(cudaMemcpyAsync(c->host_ctr, s.ctr, CTR_HOST_BYTES, cudaMemcpyDeviceToHost, st),
                 "copy counters"))
        return NCG_ECUDA;
    c->launches = launches;
    c->graph_launches = launches;
    c->last.n_pairs = b->n_pairs;
    return NCG_OK;
}

}  // namespace

extern "C" {

int ncg_abi_version(void) { return NCG_ABI_VERSION; }
const char* ncg_last_error(void) { return g_last_error.c_str(); }

int ncg_ctx_create(ncg_ctx** out, int device) {
    if (!out) return NCG_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (!cuda_ok(cudaGetDeviceCount(&ndev), "cudaGetDeviceCount")) return NCG_ECUDA;
    if (device < 0 || device >= ndev) { g_last_error = "no such device"; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice")) return NCG_ECUDA;
    ncg_ctx* c = new ncg_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    Limits lim = launch_limits();
    c->occ_thread = lim.occ_thread;
    c->occ_warp = lim.occ_warp;
    c->occ_ethread = lim.occ_ethread;
    c->occ_global = lim.occ_global;
    c->occ_smem[0] = lim.occ_smem[0];
    c->occ_smem[1] = lim.occ_smem[1];
    set_carveout(c->l1_carveout);
    c->occ_hstage = dwa::gjk_warp_stage_occupancy((uint32_t)c->hstage_cap);
    (void)f32a::gjk_warp_stage_occupancy((uint32_t)c->hstage_cap);
    c->slab_bytes[0] = (tier_bytes<2>() + 255) & ~size_t(255);
    c->slab_bytes[1] = (tier_bytes<3>() + 255) & ~size_t(255);
    c->n_slabs[0] = c->num_sms * c->occ_global;
    c->n_slabs[1] = c->num_sms;
    if (!cuda_ok(cudaMalloc(&c->slabs, c->slab_bytes[0] * c->n_slabs[0] + c->slab_bytes[1] * c->n_slabs[1]),
                 "cudaMalloc(slabs)") ||
        !cuda_ok(cudaMallocHost(&c->host_ctr, sizeof(DevCounters)), "cudaMallocHost")) {
        ncg_ctx_destroy(c);
        return NCG_ENOMEM;
    }
    memset(c->host_ctr, 0, sizeof(DevCounters));
    *out = c;
    return NCG_OK;
}

int ncg_ctx_destroy(ncg_ctx* c) {
    if (!c) return NCG_OK;
    while (!c->graphs.empty()) ncg_graph_destroy(c->graphs.back());
    cudaSetDevice(c->device);
    if (c->scratch) cudaFree(c->scratch);
    if (c->slabs) cudaFree(c->slabs);
    if (c->mlp_params) cudaFree(c->mlp_params);
    if (c->desc_buf) cudaFree(c->desc_buf);
    if (c->idir_buf) cudaFree(c->idir_buf);
    if (c->stage) cudaFree(c->stage);
    if (c->host_ctr) cudaFreeHost(c->host_ctr);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->hull_ready) cudaEventDestroy(c->hull_ready);
    for (int i = 0; i < NCG_N_MARKS; ++i)
        if (c->marks[i]) cudaEventDestroy(c->marks[i]);
    delete c;
    return NCG_OK;
}

int ncg_ctx_set_tolerance(ncg_ctx* c, int tol) {
    if (!c || (tol != NCG_TOL_REFERENCE && tol != NCG_TOL_PRECISE)) return NCG_EINVAL;
    c->tol_mode = tol;
    return NCG_OK;
}

int ncg_ctx_set_arithmetic(ncg_ctx* c, int arith) {
    if (!c || (arith != NCG_ARITH_SPLIT && arith != NCG_ARITH_F32)) return NCG_EINVAL;
    c->arith = arith;
    return NCG_OK;
}

int ncg_ctx_set_mlp_params(ncg_ctx* c, const float* params, int n) {
    if (!c || !params || n != NCG_MLP_N_PARAMS) { g_last_error = "expected NCG_MLP_N_PARAMS parameters"; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    if (!c->mlp_params && !cuda_ok(cudaMalloc(&c->mlp_params, 4 * (size_t)n), "cudaMalloc(mlp params)"))
        return NCG_ENOMEM;
    // host or device source (unified addressing)
    return cuda_ok(cudaMemcpy(c->mlp_params, params, 4 * (size_t)n, cudaMemcpyDefault), "copy mlp params") ? NCG_OK
                                                                                                          : NCG_ECUDA;
}

int ncg_ctx_set_tuning(ncg_ctx* c, int key, int value) {
    if (!c) return NCG_EINVAL;
    switch (key) {
    case NCG_TUNE_HULL_GJK_WARP:
        if (value < 0 || value > 3 + NB_HULL - 1) return NCG_EINVAL;
        c->hull_gjk_warp = value;
        return NCG_OK;
    case NCG_TUNE_GJK_BLOCKS:
        if (value < 0 || value > c->occ_thread) return NCG_EINVAL;
        c->gjk_blocks = value;
        return NCG_OK;
    case NCG_TUNE_EPA_BLOCKS:
        if (value < 0 || value > c->occ_ethread) return NCG_EINVAL;
        c->epa_blocks = value;
        return NCG_OK;
    case NCG_TUNE_L1_CARVEOUT:
        if (value < -1 || value > 100) return NCG_EINVAL;
        if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
        c->l1_carveout = value;
        return set_carveout(value) ? NCG_OK : NCG_ECUDA;
    case NCG_TUNE_HULL_EPA_WARP:
        if (value < 0 || value > 3 + NB_HULL - 1 || value == 1) return NCG_EINVAL;
        c->hull_epa_warp = value;
        return NCG_OK;
    case NCG_TUNE_HULL_LOCALITY:
        if (value < 0 || value > 1) return NCG_EINVAL;
        c->hull_locality = value;
        return NCG_OK;
    case NCG_TUNE_HULL_STAGE_MIN:
        if (value < 0 || value > 2048) return NCG_EINVAL;
        c->hstage_min = value;
        return NCG_OK;
    case NCG_TUNE_HULL_STAGE_CAP: {
        if (value < 32 || value > 2048 || value % 32 != 0) return NCG_EINVAL;
        if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
        const int occ = dwa::gjk_warp_stage_occupancy((uint32_t)value);
        (void)f32a::gjk_warp_stage_occupancy((uint32_t)value);
        if (occ <= 0) { g_last_error = "hull stage does not fit in shared memory"; return NCG_EINVAL; }
        c->hstage_cap = value;
        c->occ_hstage = occ;
        return NCG_OK;
    }
    default:
        g_last_error = "unknown tuning key";
        return NCG_EINVAL;
    }
}

int ncg_ctx_set_dispatch(ncg_ctx* c, int dispatch) {
    if (!c || (dispatch != NCG_DISPATCH_SUPPORT_MAP && dispatch != NCG_DISPATCH_QUERY)) return NCG_EINVAL;
    c->dispatch = dispatch;
    return NCG_OK;
}

int ncg_ctx_set_profiling(ncg_ctx* c, int enabled) {
    if (!c) return NCG_EINVAL;
    if (enabled && !c->marks[0]) {
        for (int i = 0; i < NCG_N_MARKS; ++i)
            if (!cuda_ok(cudaEventCreate(&c->marks[i]), "cudaEventCreate")) return NCG_ECUDA;
    }
    c->profiling = enabled ? 1 : 0;
    return NCG_OK;
}

int ncg_get_stage_ms(ncg_ctx* c, float* ms, int n_max) {
    if (!c || !ms) return NCG_EINVAL;
    for (int i = 0; i < n_max; ++i) ms[i] = 0.0f;
    if (!c->profiling || c->n_marks < 2) return 0;
    if (!cuda_ok(cudaEventSynchronize(c->marks[c->n_marks - 1]), "cudaEventSynchronize")) return NCG_ECUDA;
    int wrote = 0;
    for (int i = 1; i < c->n_marks; ++i) {
        int stage = c->mark_stage[i];
        float t = 0.0f;
        cudaEventElapsedTime(&t, c->marks[i - 1], c->marks[i]);
        if (stage >= 0 && stage < n_max) {
            ms[stage] += t;
            if (stage + 1 > wrote) wrote = stage + 1;
        }
    }
    return wrote;
}

int ncg_ctx_set_warm_start(ncg_ctx* c, int w) {
    if (!c || w < NCG_WARM_NONE || w > NCG_WARM_MLP) return NCG_EINVAL;
    c->warm = w;
    return NCG_OK;
}

int ncg_sync(ncg_ctx* c, void* stream) {
    if (!c) return NCG_EINVAL;
    if (!cuda_ok(cudaStreamSynchronize((cudaStream_t)stream), "cudaStreamSynchronize")) return NCG_ECUDA;
    return NCG_OK;
}

int ncg_get_stats(ncg_ctx* c, ncg_stats* out) {
    if (!c || !out) return NCG_EINVAL;
    // host_ctr was filled by an asynchronous copy at the end of the last call;
    // the caller synchronises the stream before reading the statistics.
    out->n_pairs = c->last.n_pairs;
    out->n_epa = c->host_ctr->n_items;
    out->n_epa_overflow = c->host_ctr->epa_count[Q_WARP_LONG] + c->host_ctr->epa_count[Q_WARP];
    out->gjk_iters = c->host_ctr->gjk_iters;
    out->epa_iters = c->host_ctr->epa_iters;
    out->n_epa_thread = c->host_ctr->epa_count[0] + c->host_ctr->epa_count[Q_THREAD_HULL];
    out->kernels_launched = c->launches;
    out->flags = (c->host_ctr->mlp_err & 1u) | ((c->host_ctr->stage_err & 1u) << 1);
    return NCG_OK;
}

int ncg_contact_batch(ncg_ctx* c, const ncg_batch* b, float prediction, ncg_contact* out, uint8_t* has_contact,
                      float* out_dir, uint32_t* status, uint32_t* iters, void* stream) {
    if (c && b && b->n_pairs == 0) return NCG_OK;
    if (!out || !has_contact) { g_last_error = "null output"; return NCG_EINVAL; }
    Outputs o{out, has_contact, out_dir, nullptr, nullptr, status, iters};
    return run_query(c, b, Q_CONTACT, prediction, o, (cudaStream_t)stream);
}

struct ncg_graph {
    ncg_ctx* ctx;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

int ncg_contact_graph_create(ncg_ctx* c, const ncg_batch* b, float prediction, ncg_contact* out, uint8_t* has_contact,
                             float* out_dir, uint32_t* status, uint32_t* iters, ncg_graph** g) {
    if (!g) return NCG_EINVAL;
    *g = nullptr;
    if (!c || !b || !out || !has_contact) { g_last_error = "null argument"; return NCG_EINVAL; }
    if (b->n_pairs == 0) { g_last_error = "empty batch"; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    // everything that allocates happens before the capture
    if (!ensure_scratch(c, b->n_pairs)) return NCG_ENOMEM;
    if (c->warm == NCG_WARM_MLP) {
        int rc0 = ensure_mlp_buffers(c, b);
        if (rc0 != NCG_OK) return rc0;
    }
    cudaStream_t cs;
    if (!cuda_ok(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate")) return NCG_ECUDA;
    const int prof = c->profiling;
    c->profiling = 0;
    Outputs o{out, has_contact, out_dir, nullptr, nullptr, status, iters};
    int rc = NCG_OK;
    cudaGraph_t graph = nullptr;
    if (!cuda_ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture")) rc = NCG_ECUDA;
    if (rc == NCG_OK) {
        rc = run_query(c, b, Q_CONTACT, prediction, o, cs);
        cudaError_t e = cudaStreamEndCapture(cs, &graph);
        if (rc == NCG_OK && !cuda_ok(e, "cudaStreamEndCapture")) rc = NCG_ECUDA;
    }
    c->profiling = prof;
    cudaGraphExec_t exec = nullptr;
    if (rc == NCG_OK && !cuda_ok(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate")) rc = NCG_ECUDA;
    cudaStreamDestroy(cs);
    if (rc != NCG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    ncg_graph* h = new ncg_graph{c, graph, exec};
    c->graphs.push_back(h);
    *g = h;
    return NCG_OK;
}

int ncg_graph_launch(ncg_graph* g, void* stream) {
    if (!g) return NCG_EINVAL;
    if (!cuda_ok(cudaSetDevice(g->ctx->device), "cudaSetDevice")) return NCG_ECUDA;
    if (!cuda_ok(cudaGraphLaunch(g->exec, (cudaStream_t)stream), "cudaGraphLaunch")) return NCG_ECUDA;
    g->ctx->launches = g->ctx->graph_launches;
    return NCG_OK;
}

int ncg_graph_destroy(ncg_graph* g) {
    if (!g) return NCG_OK;
    auto& v = g->ctx->graphs;
    for (size_t i = 0; i < v.size(); ++i)
        if (v[i] == g) { v.erase(v.begin() + (long)i); break; }
    cudaSetDevice(g->ctx->device);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return NCG_OK;
}

int ncg_distance_batch(ncg_ctx* c, const ncg_batch* b, float* out_dist, uint32_t* status, uint32_t* iters,
                       void* stream) {
    if (c && b && b->n_pairs == 0) return NCG_OK;
    if (!out_dist) { g_last_error = "null output"; return NCG_EINVAL; }
    Outputs o{nullptr, nullptr, nullptr, out_dist, nullptr, status, iters};
    return run_query(c, b, Q_DISTANCE, 0.0f, o, (cudaStream_t)stream);
}

int ncg_proximity_batch(ncg_ctx* c, const ncg_batch* b, float margin, uint8_t* out_prox, float* out_sep_axis,
                        uint32_t* status, uint32_t* iters, void* stream) {
    if (!(margin >= 0.0f)) { g_last_error = "The proximity margin must be positive or zero."; return NCG_EINVAL; }
    if (c && b && b->n_pairs == 0) return NCG_OK;
    if (!out_prox) { g_last_error = "null output"; return NCG_EINVAL; }
    Outputs o{nullptr, out_prox, out_sep_axis, nullptr, nullptr, status, iters};
    return run_query(c, b, Q_PROXIMITY, margin, o, (cudaStream_t)stream);
}

int ncg_closest_points_batch(ncg_ctx* c, const ncg_batch* b, float prediction, uint8_t* out_tag, float* out_points,
                             uint32_t* status, uint32_t* iters, void* stream) {
    if (c && b && b->n_pairs == 0) return NCG_OK;
    if (!out_tag) { g_last_error = "null output"; return NCG_EINVAL; }
    Outputs o{nullptr, out_tag, nullptr, nullptr, out_points, status, iters};
    return run_query(c, b, Q_CLOSEST, prediction, o, (cudaStream_t)stream);
}

int ncg_time_of_impact_batch(ncg_ctx* c, const ncg_batch* b, const float* vel1, const float* vel2, float max_toi,
                             float target_distance, ncg_toi* out, uint8_t* has_toi, uint32_t* status, uint32_t* iters,
                             void* stream) {
    if (!(max_toi >= 0.0f) || !(target_distance >= 0.0f)) {
        g_last_error = "max_toi and target_distance must be >= 0";
        return NCG_EINVAL;
    }
    if (!c || !b) { g_last_error = "null context or batch"; return NCG_EINVAL; }
    if (b->n_pairs == 0) return NCG_OK;
    if (b->n_pairs > 0xffffffffull) { g_last_error = "more than 2^32-1 pairs"; return NCG_EINVAL; }
    if (!b->shapes || !b->m1 || !b->m2 || !b->g1 || !b->g2 || !vel1 || !vel2 || !out || !has_toi || !status) {
        g_last_error = "null required pointer";
        return NCG_EINVAL;
    }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    if (!ensure_scratch(c, b->n_pairs)) return NCG_ENOMEM;
    const Scratch s = carve_scratch(c);
    const Tol tol = make_tol(c->tol_mode);
    const cudaStream_t st = (cudaStream_t)stream;
    if (!cuda_ok(cudaMemsetAsync(s.ctr, 0, sizeof(DevCounters), st), "memset counters")) return NCG_ECUDA;
    uint32_t launches = 0;
    // the TOI counters and the refinement queue live in the EPA item area
    // (unused here; 160 bytes per pair); the ray-cast iterations are summed
    // into the statistics' GJK iteration count
    int rc = toi_launch(*b, tol, c->dispatch, vel1, vel2, max_toi, target_distance, out, has_toi, status, iters,
                        ToiScratch{s.bucket, s.sorted, s.items, reinterpret_cast<char*>(s.items) + 512,
                                   &s.ctr->gjk_iters},
                        c->num_sms, st, &launches);
    if (rc != NCG_OK) return rc;
    if (!cuda_ok(cudaMemcpyAsync(c->host_ctr, s.ctr, CTR_HOST_BYTES, cudaMemcpyDeviceToHost, st),
                 "copy counters"))
        return NCG_ECUDA;
    c->launches = launches;
    c->graph_launches = launches;
    c->last = ncg_stats{};
    c->last.n_pairs = b->n_pairs;
    return NCG_OK;
}

int ncg_ray_cast_batch(ncg_ctx* c, const ncg_batch* b, const float* rays, float max_toi, int solid, float* out_toi,
                       float* out_normal, uint8_t* has_hit, uint32_t* status, uint32_t* iters, void* stream) {
    if (!(max_toi >= 0.0f)) {
        g_last_error = "max_toi must be >= 0";
        return NCG_EINVAL;
    }
    if (!c || !b) { g_last_error = "null context or batch"; return NCG_EINVAL; }
    if (b->n_pairs == 0) return NCG_OK;
    if (b->n_pairs > 0xffffffffull) { g_last_error = "more than 2^32-1 rays"; return NCG_EINVAL; }
    if (!b->shapes || !b->m1 || !b->g1 || !rays || !out_toi || !has_hit || !status) {
        g_last_error = "null required pointer";
        return NCG_EINVAL;
    }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    if (!ensure_scratch(c, b->n_pairs)) return NCG_ENOMEM;
    const Scratch s = carve_scratch(c);
    const Tol tol = make_tol(c->tol_mode);
    const cudaStream_t st = (cudaStream_t)stream;
    if (!cuda_ok(cudaMemsetAsync(s.ctr, 0, sizeof(DevCounters), st), "memset counters")) return NCG_ECUDA;
    uint32_t launches = 0;
    int rc = ray_launch(*b, tol, rays, max_toi, solid, out_toi, out_normal, has_hit, status, iters,
                        ToiScratch{s.bucket, s.sorted, s.items, reinterpret_cast<char*>(s.items) + 512,
                                   &s.ctr->gjk_iters},
                        c->num_sms, st, &launches);
    if (rc != NCG_OK) return rc;
    if (!cuda_ok(cudaMemcpyAsync(c->host_ctr, s.ctr, CTR_HOST_BYTES, cudaMemcpyDeviceToHost, st),
                 "copy counters"))
        return NCG_ECUDA;
    c->launches = launches;
    c->graph_launches = launches;
    c->last = ncg_stats{};
    c->last.n_pairs = b->n_pairs;
    return NCG_OK;
}

int ncg_manifold_batch(ncg_ctx* c, const ncg_batch* b, float prediction, float angular1, float angular2,
                       ncg_contact* contact, uint8_t* has_contact, float* out_dir, ncg_manifold* out, uint32_t* status,
                       void* stream) {
    return ncg_manifold_batch_hulls(c, b, nullptr, prediction, angular1, angular2, contact, has_contact, out_dir, out,
                                    status, stream);
}

int ncg_manifold_batch_hulls(ncg_ctx* c, const ncg_batch* b, const ncg_hull_topology* topology, float prediction,
                             float angular1, float angular2, ncg_contact* contact, uint8_t* has_contact,
                             float* out_dir, ncg_manifold* out, uint32_t* status, void* stream) {
    if (!(prediction >= 0.0f) || !(angular1 >= 0.0f) || !(angular2 >= 0.0f)) {
        g_last_error = "the contact prediction must be >= 0";
        return NCG_EINVAL;
    }
    if (c && b && b->n_pairs == 0) return NCG_OK;
    if (!contact || !has_contact || !out || !status) { g_last_error = "null output"; return NCG_EINVAL; }
    if (!c) { g_last_error = "null context"; return NCG_EINVAL; }
    // the generator calls contact_support_map_support_map_with_params for every pair
    const int dispatch = c->dispatch;
    c->dispatch = NCG_DISPATCH_SUPPORT_MAP;
    Outputs o{contact, has_contact, out_dir, nullptr, nullptr, status, nullptr};
    const cudaStream_t st = (cudaStream_t)stream;
    int rc = run_query(c, b, Q_CONTACT, prediction, o, st);
    c->dispatch = dispatch;
    if (rc != NCG_OK) return rc;
    const ncg::ManifoldParams mp{prediction, std::cos(angular1), std::sin(angular1), std::cos(angular2),
                                 std::sin(angular2)};
    ncg::HullTopo topo{};
    if (topology) {
        if (topology->n_shapes < b->n_shapes || topology->n_hull_points < b->n_hull_points || !topology->shape) {
            g_last_error = "ncg_manifold_batch_hulls: the topology covers fewer shapes or hull points than the batch";
            return NCG_EINVAL;
        }
        topo = ncg::HullTopo{topology->shape,       topology->face_normal, topology->face_range,
                             topology->face_vertex, topology->face_edge,   topology->edge_vertex,
                             topology->edge_dir,    topology->vertex_range, topology->vertex_face,
                             topology->vertex_edge};
    }
    rc = ncg::manifold_launch(*b, contact, has_contact, mp, topo, out, status, c->num_sms, st);
    if (rc == NCG_OK) c->launches += 1;
    return rc;
}

int ncg_aabb_batch(ncg_ctx* c, const ncg_batch* b, float* out_aabbs, uint32_t* status, void* stream) {
    if (!c || !b) { g_last_error = "null context or batch"; return NCG_EINVAL; }
    if (b->n_pairs == 0) return NCG_OK;
    if (!b->shapes || !b->m1 || !b->g1 || !out_aabbs) { g_last_error = "null required pointer"; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    int rc = aabb_launch(*b, out_aabbs, status, c->num_sms, (cudaStream_t)stream);
    if (rc == NCG_OK) c->launches = 1;
    return rc;
}

struct ncg_broad_phase {
    ncg::BroadPhaseState* s;
};

int ncg_bp_create(ncg_ctx* c, float margin, ncg_broad_phase** out) {
    if (!c || !out) { g_last_error = "null context or output"; return NCG_EINVAL; }
    if (!(margin >= 0.0f)) { g_last_error = "The loosening margin must be positive."; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    ncg::BroadPhaseState* s = nullptr;
    int rc = ncg::bp_create(margin, c->device, &s);
    if (rc != NCG_OK) return rc;
    *out = new ncg_broad_phase{s};
    return NCG_OK;
}

int ncg_bp_update(ncg_broad_phase* bp, const float* aabbs, uint32_t n, void* stream) {
    if (!bp) { g_last_error = "null broad phase"; return NCG_EINVAL; }
    if (n > 0 && !aabbs) { g_last_error = "null boxes"; return NCG_EINVAL; }
    if (n > (1u << 30)) { g_last_error = "more than 2^30 proxies"; return NCG_EINVAL; }
    return ncg::bp_update(bp->s, aabbs, n, (cudaStream_t)stream);
}

int ncg_bp_results(ncg_broad_phase* bp, uint64_t* n_pairs, uint64_t* n_started, uint64_t* n_stopped,
                   const uint32_t** pairs, const uint32_t** started, const uint32_t** stopped) {
    if (!bp) { g_last_error = "null broad phase"; return NCG_EINVAL; }
    ncg::bp_results(bp->s, n_pairs, n_started, n_stopped, pairs, started, stopped);
    return NCG_OK;
}

int ncg_bp_copy(ncg_broad_phase* bp, uint32_t* pairs, uint32_t* started, uint32_t* stopped, void* stream) {
    if (!bp) { g_last_error = "null broad phase"; return NCG_EINVAL; }
    uint64_t n[3];
    const uint32_t* src[3];
    ncg::bp_results(bp->s, &n[0], &n[1], &n[2], &src[0], &src[1], &src[2]);
    uint32_t* dst[3] = {pairs, started, stopped};
    for (int k = 0; k < 3; ++k) {
        if (!dst[k] || n[k] == 0) continue;
        if (!cuda_ok(cudaMemcpyAsync(dst[k], src[k], 8 * n[k], cudaMemcpyDefault, (cudaStream_t)stream),
                     "ncg_bp_copy"))
            return NCG_ECUDA;
    }
    return NCG_OK;
}

int ncg_gather_pairs(ncg_ctx* c, const ncg_pose* poses, const uint32_t* shape_ids, const uint32_t* pairs,
                     uint64_t n, ncg_pose* m1, uint32_t* g1, ncg_pose* m2, uint32_t* g2, void* stream) {
    if (!c) { g_last_error = "null context"; return NCG_EINVAL; }
    if (n == 0) return NCG_OK;
    if (!poses || !shape_ids || !pairs || !m1 || !g1 || !m2 || !g2) {
        g_last_error = "null required pointer";
        return NCG_EINVAL;
    }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    return ncg::gather_launch(poses, shape_ids, pairs, n, m1, g1, m2, g2, c->num_sms, (cudaStream_t)stream);
}

int ncg_bp_destroy(ncg_broad_phase* bp) {
    if (!bp) return NCG_OK;
    ncg::bp_destroy(bp->s);
    delete bp;
    return NCG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ host-memory entry points
namespace {

struct HostRun {
    ncg_batch dev;
    char* out;
};

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// Copies a host batch into the context's staging buffer; returns the device batch
// and a pointer to `out_bytes` of device output space after the inputs.
int stage_batch(ncg_ctx* c, const ncg_batch* h, size_t out_bytes, cudaStream_t st, HostRun& hr) {
    const uint64_t n = h->n_pairs;
    size_t need = al(sizeof(ncg_shape) * h->n_shapes) + al(16 * h->n_hull_points) + 2 * al(sizeof(ncg_pose) * n) +
                  2 * al(4 * n) + (h->init_dir ? al(12 * n) : 0) + al(out_bytes);
    if (need > c->stage_cap) {
        if (c->stage) cudaFree(c->stage);
        c->stage = nullptr;
        if (!cuda_ok(cudaMalloc(&c->stage, need), "cudaMalloc(stage)")) return NCG_ENOMEM;
        c->stage_cap = need;
    }
    char* p = c->stage;
    ncg_batch d = *h;
    auto put = [&](const void* src, size_t bytes, cudaStream_t s) -> char* {
        char* dst = p;
        if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
        p += al(bytes);
        return dst;
    };
    // The small arrays first, on st; then the hull points (most of the bytes)
    // on the copy stream once those are done (copies in one direction share
    // the copy engines in issue order, so the query's first kernels would
    // otherwise wait behind the hull points).  The query waits for hull_ready
    // before its first kernel that reads hull points.
    char* hull_dst = p;
    p += al(16 * h->n_hull_points);
    d.shapes = (const ncg_shape*)put(h->shapes, sizeof(ncg_shape) * h->n_shapes, st);
    d.m1 = (const ncg_pose*)put(h->m1, sizeof(ncg_pose) * n, st);
    d.m2 = (const ncg_pose*)put(h->m2, sizeof(ncg_pose) * n, st);
    d.g1 = (const uint32_t*)put(h->g1, 4 * n, st);
    d.g2 = (const uint32_t*)put(h->g2, 4 * n, st);
    d.init_dir = h->init_dir ? (const float*)put(h->init_dir, 12 * n, st) : nullptr;
    if (!cuda_ok(cudaEventRecord(c->hull_ready, st), "cudaEventRecord") ||
        !cuda_ok(cudaStreamWaitEvent(c->copy_stream, c->hull_ready, 0), "cudaStreamWaitEvent"))
        return NCG_ECUDA;
    if (h->n_hull_points)
        cudaMemcpyAsync(hull_dst, h->hull_points, 16 * h->n_hull_points, cudaMemcpyHostToDevice, c->copy_stream);
    d.hull_points = (const float*)hull_dst;
    if (!cuda_ok(cudaEventRecord(c->hull_ready, c->copy_stream), "cudaEventRecord")) return NCG_ECUDA;
    hr.dev = d;
    hr.out = p;
    return cuda_ok(cudaGetLastError(), "stage copies") ? NCG_OK : NCG_ECUDA;
}

// Ends a host entry point: the stream also waits for the hull-point copy (so
// that no copy from the caller's buffers is in flight when the call returns,
// whatever the query read), then the host waits for the stream.
int host_finish(ncg_ctx* c, cudaStream_t st, int rc, const char* what) {
    cudaStreamWaitEvent(st, c->hull_ready, 0);
    const bool ok = cuda_ok(cudaStreamSynchronize(st), what);
    return rc != NCG_OK ? rc : (ok ? NCG_OK : NCG_ECUDA);
}

cudaStream_t host_stream(ncg_ctx* c) {
    if (!c->own_stream) cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (!c->copy_stream) cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking);
    if (!c->hull_ready) cudaEventCreateWithFlags(&c->hull_ready, cudaEventDisableTiming);
    return c->own_stream;
}

}  // namespace

extern "C" {

int ncg_contact_batch_host(ncg_ctx* c, const ncg_batch* b, float prediction, ncg_contact* out, uint8_t* has_contact,
                           float* out_dir, uint32_t* status) {
    if (!c || !b || !out || !has_contact || !status) return NCG_EINVAL;
    if (b->n_pairs == 0) return NCG_OK;
    cudaSetDevice(c->device);
    cudaStream_t st = host_stream(c);
    const uint64_t n = b->n_pairs;
    size_t ob = al(40 * n) + al(n) + al(12 * n) + al(4 * n);
    HostRun hr;
    int rc = stage_batch(c, b, ob, st, hr);
    if (rc) return host_finish(c, st, rc, "contact_batch_host");
    ncg_contact* dc = (ncg_contact*)hr.out;
    uint8_t* dt = (uint8_t*)(hr.out + al(40 * n));
    float* dd = (float*)(hr.out + al(40 * n) + al(n));
    uint32_t* ds = (uint32_t*)(hr.out + al(40 * n) + al(n) + al(12 * n));
    Outputs o{dc, dt, out_dir ? dd : nullptr, nullptr, nullptr, ds, nullptr};
    rc = run_query(c, &hr.dev, Q_CONTACT, prediction, o, st, c->hull_ready);
    if (rc) return host_finish(c, st, rc, "contact_batch_host");
    cudaMemcpyAsync(out, dc, 40 * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(has_contact, dt, n, cudaMemcpyDeviceToHost, st);
    if (out_dir) cudaMemcpyAsync(out_dir, dd, 12 * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(status, ds, 4 * n, cudaMemcpyDeviceToHost, st);
    return host_finish(c, st, NCG_OK, "contact_batch_host");
}

int ncg_distance_batch_host(ncg_ctx* c, const ncg_batch* b, float* out_dist, uint32_t* status) {
    if (!c || !b || !out_dist || !status) return NCG_EINVAL;
    if (b->n_pairs == 0) return NCG_OK;
    cudaSetDevice(c->device);
    cudaStream_t st = host_stream(c);
    const uint64_t n = b->n_pairs;
    HostRun hr;
    int rc = stage_batch(c, b, al(4 * n) + al(4 * n), st, hr);
    if (rc) return host_finish(c, st, rc, "distance_batch_host");
    float* dd = (float*)hr.out;
    uint32_t* ds = (uint32_t*)(hr.out + al(4 * n));
    Outputs o{nullptr, nullptr, nullptr, dd, nullptr, ds, nullptr};
    rc = run_query(c, &hr.dev, Q_DISTANCE, 0.0f, o, st, c->hull_ready);
    if (rc) return host_finish(c, st, rc, "distance_batch_host");
    cudaMemcpyAsync(out_dist, dd, 4 * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(status, ds, 4 * n, cudaMemcpyDeviceToHost, st);
    return host_finish(c, st, NCG_OK, "distance_batch_host");
}

int ncg_proximity_batch_host(ncg_ctx* c, const ncg_batch* b, float margin, uint8_t* out_prox, float* out_sep_axis,
                             uint32_t* status) {
    if (!c || !b || !out_prox || !status) return NCG_EINVAL;
    if (!(margin >= 0.0f)) { g_last_error = "The proximity margin must be positive or zero."; return NCG_EINVAL; }
    if (b->n_pairs == 0) return NCG_OK;
    cudaSetDevice(c->device);
    cudaStream_t st = host_stream(c);
    const uint64_t n = b->n_pairs;
    HostRun hr;
    int rc = stage_batch(c, b, al(n) + al(12 * n) + al(4 * n), st, hr);
    if (rc) return host_finish(c, st, rc, "proximity_batch_host");
    uint8_t* dt = (uint8_t*)hr.out;
    float* dd = (float*)(hr.out + al(n));
    uint32_t* ds = (uint32_t*)(hr.out + al(n) + al(12 * n));
    Outputs o{nullptr, dt, out_sep_axis ? dd : nullptr, nullptr, nullptr, ds, nullptr};
    rc = run_query(c, &hr.dev, Q_PROXIMITY, margin, o, st, c->hull_ready);
    if (rc) return host_finish(c, st, rc, "proximity_batch_host");
    cudaMemcpyAsync(out_prox, dt, n, cudaMemcpyDeviceToHost, st);
    if (out_sep_axis) cudaMemcpyAsync(out_sep_axis, dd, 12 * n, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(status, ds, 4 * n, cudaMemcpyDeviceToHost, st);
    return host_finish(c, st, NCG_OK, "proximity_batch_host");
}

}  // extern "C"

// ------------------------------------------------------------------ no-allocation entry point
// ncg_contact_batch_noalloc runs the contact pipeline on a fixed scratch array
// in the library's device image instead of context-owned allocations.  Layout
// of the array: counters (512 B), EPA work items, routing lists and stage
// queues (7 x 4 B per pair), one tier-D EPA slab.  The counters hold the
// pair sort's per-key counts (about 580 KB).
namespace {
constexpr uint64_t NA_MAX_PAIRS = NCG_NOALLOC_MAX_PAIRS;
constexpr size_t NA_SLAB_BYTES =
    (EpaStore::bytes(EpaTier<3>::VC, EpaTier<3>::FC, EpaTier<3>::SC, EpaTier<3>::TC, EpaTier<3>::FC) + 255) &
    ~size_t(255);
constexpr size_t NA_ITEMS_BYTES = sizeof(EpaItem) * NA_MAX_PAIRS;
constexpr size_t NA_LISTS_BYTES = (2 + N_EPA_QUEUES) * 4 * NA_MAX_PAIRS;
constexpr size_t NA_BYTES = CTR_SLOT + NA_ITEMS_BYTES + NA_LISTS_BYTES + NA_SLAB_BYTES;
}  // namespace

// Host code must not use this name as an address: it is only a host-side stand-in.
static_assert(NA_BYTES == NCG_NOALLOC_SCRATCH_BYTES, "ncg.h states the no-allocation scratch size");
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {
struct NoallocDevice {
    bool ready;
    char* base;  // device address of g_noalloc_scratch on this device
    int num_sms;
    Limits lim;
};
std::mutex g_noalloc_mu;
constexpr int NA_MAX_DEVICES = 64;
NoallocDevice g_noalloc[NA_MAX_DEVICES] = {};

// One-time set-up for the current device: the array's device address and the
// launch limits.  No allocation.
int noalloc_setup(int dev, NoallocDevice& out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocDevice& d = g_noalloc[dev];
    if (!d.ready) {
        void* p = nullptr;
        if (!cuda_ok(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(noalloc scratch)"))
            return NCG_ECUDA;
        d.base = (char*)p;
        if (!cuda_ok(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev), "device attribute"))
            return NCG_ECUDA;
        d.lim = launch_limits();
        if (!cuda_ok(cudaGetLastError(), "noalloc set-up")) return NCG_ECUDA;
        d.ready = true;
    }
    out = d;
    return NCG_OK;
}
}  // namespace

extern "C" int ncg_contact_batch_noalloc(const ncg_batch* b, float prediction, int tolerance, ncg_contact* out,
                                         uint8_t* has_contact, float* out_dir, uint32_t* status, void* stream) {
    if (!b) { g_last_error = "null batch"; return NCG_EINVAL; }
    if (b->n_pairs > NA_MAX_PAIRS) {
        g_last_error = "ncg_contact_batch_noalloc: batch of " + std::to_string(b->n_pairs) +
                       " pairs exceeds NCG_NOALLOC_MAX_PAIRS (" + std::to_string(NA_MAX_PAIRS) + ")";
        return NCG_EINVAL;
    }
    if (tolerance != NCG_TOL_REFERENCE && tolerance != NCG_TOL_PRECISE) {
        g_last_error = "unknown tolerance set";
        return NCG_EINVAL;
    }
    if (b->n_pairs == 0) return NCG_OK;
    if (!out || !has_contact || !status || !b->shapes || !b->m1 || !b->m2 || !b->g1 || !b->g2) {
        g_last_error = "null required pointer";
        return NCG_EINVAL;
    }
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return NCG_ECUDA;
    if (dev < 0 || dev >= NA_MAX_DEVICES) { g_last_error = "device index out of range"; return NCG_EINVAL; }
    cudaStream_t st = (cudaStream_t)stream;
    int sdev = -1;
    if (!cuda_ok(cudaStreamGetDevice(st, &sdev), "cudaStreamGetDevice")) return NCG_EINVAL;
    if (sdev != dev) {
        g_last_error = "ncg_contact_batch_noalloc: the stream belongs to device " + std::to_string(sdev) +
                       ", not to the current device " + std::to_string(dev);
        return NCG_EINVAL;
    }
    NoallocDevice d;
    int rc = noalloc_setup(dev, d);
    if (rc) return rc;

    Scratch s;
    char* p = d.base;
    s.ctr = (DevCounters*)p; p += CTR_SLOT;
    s.items = (EpaItem*)p; p += NA_ITEMS_BYTES;
    s.bucket = (uint8_t*)p; p += 4 * NA_MAX_PAIRS;
    s.sub = (uint16_t*)(s.bucket + 2 * NA_MAX_PAIRS);
    s.loc_shift = 32;
    s.sorted = (uint32_t*)p; p += 4 * NA_MAX_PAIRS;
    for (int q = 0; q < N_EPA_QUEUES; ++q) { s.queue[q] = (uint32_t*)p; p += 4 * NA_MAX_PAIRS; }
    s.slabs[0] = p;
    s.slab_bytes[0] = NA_SLAB_BYTES;
    s.n_slabs[0] = 1;
    s.slabs[1] = nullptr;
    s.slab_bytes[1] = 0;
    s.n_slabs[1] = 0;
    s.spill = nullptr;  // no spill records: overflowing pairs restart from GJK's simplex
    s.spill_of = nullptr;
    s.spill_bytes = 0;
    s.spill_cap = 0;

    QueryParams qp;
    qp.query = Q_CONTACT;
    qp.dispatch = NCG_DISPATCH_SUPPORT_MAP;
    qp.use_init_dir = b->init_dir ? 1 : 0;
    qp.gjk_max_iter = 10000;
    qp.epa_max_iter = 10000;
    qp.param = dw_split((double)prediction);
    qp.tol = make_tol(tolerance);
    Outputs o{out, has_contact, out_dir, nullptr, nullptr, status, nullptr};
    ncg_batch bb = *b;

    // The array keeps the previous call's contents: reset the counters and queues' heads.
    if (!cuda_ok(cudaMemsetAsync(s.ctr, 0, sizeof(DevCounters), st), "memset noalloc counters")) return NCG_ECUDA;
    dwa::gjk_launch_sort(bb, qp, o, s, st);
    dwa::gjk_launch_thread(d.num_sms * d.lim.occ_thread, bb, qp, o, s, 0, 0, 0, 0, st);
    dwa::gjk_launch_thread(d.num_sms * d.lim.occ_thread, bb, qp, o, s, 1, 0, 0, 0, st);
    dwa::epa_launch_thread(d.num_sms * d.lim.occ_ethread, bb, qp, o, s, 0, st);
    // warp stages in shared memory (128, then 1280 vertices), then the one global slab
    dwa::epa_launch_warp(d.num_sms * d.lim.occ_smem[0], tier_bytes<1>(), bb, qp, o, s, caps<1>(Q_WARP_LONG, Q_WARP, 3, -1),
                         st);
    dwa::epa_launch_warp(d.num_sms * d.lim.occ_smem[1], tier_bytes<2>(), bb, qp, o, s, caps<2>(3, -1, 4, -1), st);
    TierCaps last = caps<3>(4, -1, -1, 0);
    last.HC = last.FC;  // the slab above: the double-word build's heap never holds more than FC entries
    dwa::epa_launch_warp(1, 0, bb, qp, o, s, last, st);
    return cuda_ok(cudaGetLastError(), "noalloc kernel launch") ? NCG_OK : NCG_ECUDA;
}

// ------------------------------------------------------------------ autotuner
namespace {

// Order-independent digest of a byte buffer: the sum over 32-bit words of a
// 64-bit mix (splitmix64's finaliser) of (word index, word).  A tail that is
// not a whole word is zero-padded.
__global__ void k_digest(const uint8_t* p, uint64_t nbytes, unsigned long long* out) {
    const uint64_t nw = (nbytes + 3) / 4;
    unsigned long long acc = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t w = 0;
        if (4 * i + 4 <= nbytes) w = *reinterpret_cast<const uint32_t*>(p + 4 * i);
        else
            for (uint64_t k = 4 * i; k < nbytes; ++k) w |= (uint32_t)p[k] << (8 * (k - 4 * i));
        uint64_t z = (i << 32) ^ w;
        z += 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        acc += z ^ (z >> 31);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31u) == 0) atomicAdd(out, acc);
}

struct TuneOutputs {
    char* buf = nullptr;
    Outputs o{};
    std::vector<std::pair<const uint8_t*, uint64_t>> parts;  // what the digest covers
    unsigned long long* digest = nullptr;                    // 8-byte device slot
};

int tune_alloc(int query, uint64_t n, TuneOutputs& t) {
    const uint64_t sz[7] = {query == Q_CONTACT ? 40 * n : 0, 1 * n, 12 * n, 4 * n, 24 * n, 4 * n, 8};
    uint64_t off[7], total = 0;
    for (int k = 0; k < 7; ++k) { off[k] = total; total += (sz[k] + 255) & ~uint64_t(255); }
    if (!cuda_ok(cudaMalloc(&t.buf, total), "cudaMalloc(autotune outputs)")) return NCG_ENOMEM;
    char* b = t.buf;
    t.digest = (unsigned long long*)(b + off[6]);
    t.o = Outputs{};
    t.o.status = (uint32_t*)(b + off[3]);
    t.parts.push_back({(const uint8_t*)t.o.status, 4 * n});
    switch (query) {
    case Q_CONTACT:
        t.o.contact = (ncg_contact*)(b + off[0]);
        t.o.tag = (uint8_t*)(b + off[1]);
        t.o.dir = (float*)(b + off[2]);
        t.parts.push_back({(const uint8_t*)t.o.contact, 40 * n});
        t.parts.push_back({t.o.tag, n});
        t.parts.push_back({(const uint8_t*)t.o.dir, 12 * n});
        break;
    case Q_DISTANCE:
        t.o.value = (float*)(b + off[5]);
        t.parts.push_back({(const uint8_t*)t.o.value, 4 * n});
        break;
    case Q_PROXIMITY:
        t.o.tag = (uint8_t*)(b + off[1]);
        t.o.dir = (float*)(b + off[2]);
        t.parts.push_back({t.o.tag, n});
        t.parts.push_back({(const uint8_t*)t.o.dir, 12 * n});
        break;
    default:
        t.o.tag = (uint8_t*)(b + off[1]);
        t.o.points = (float*)(b + off[4]);
        t.parts.push_back({t.o.tag, n});
        t.parts.push_back({(const uint8_t*)t.o.points, 24 * n});
    }
    return NCG_OK;
}

// Times one configuration: one untimed call, then `reps` timed calls; the
// fastest is its time.  *digest covers the outputs of the last call.
int tune_time(ncg_ctx* c, const ncg_batch* b, int query, float param, int reps, TuneOutputs& t, cudaStream_t st,
              cudaEvent_t e0, cudaEvent_t e1, float* ms, unsigned long long* digest) {
    float best = 0.0f;
    for (int r = 0; r <= reps; ++r) {
        if (!cuda_ok(cudaEventRecord(e0, st), "cudaEventRecord")) return NCG_ECUDA;
        int rc = run_query(c, b, query, param, t.o, st);
        if (rc != NCG_OK) return rc;
        if (!cuda_ok(cudaEventRecord(e1, st), "cudaEventRecord") ||
            !cuda_ok(cudaEventSynchronize(e1), "cudaEventSynchronize"))
            return NCG_ECUDA;
        float m = 0.0f;
        if (!cuda_ok(cudaEventElapsedTime(&m, e0, e1), "cudaEventElapsedTime")) return NCG_ECUDA;
        if (r > 0 && (r == 1 || m < best)) best = m;
    }
    unsigned long long* slot = t.digest;
    if (!cuda_ok(cudaMemsetAsync(slot, 0, 8, st), "memset digest")) return NCG_ECUDA;
    for (auto& p : t.parts) k_digest<<<c->num_sms * 4, 256, 0, st>>>(p.first, p.second, slot);
    unsigned long long h = 0;
    if (!cuda_ok(cudaMemcpyAsync(&h, slot, 8, cudaMemcpyDeviceToHost, st), "copy digest") ||
        !cuda_ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return NCG_ECUDA;
    *ms = best;
    *digest = h;
    return NCG_OK;
}

}  // namespace

extern "C" {

int ncg_ctx_get_tuning(ncg_ctx* c, int key, int* value) {
    if (!c || !value) return NCG_EINVAL;
    switch (key) {
    case NCG_TUNE_HULL_GJK_WARP: *value = c->hull_gjk_warp; return NCG_OK;
    case NCG_TUNE_GJK_BLOCKS: *value = c->gjk_blocks; return NCG_OK;
    case NCG_TUNE_EPA_BLOCKS: *value = c->epa_blocks; return NCG_OK;
    case NCG_TUNE_L1_CARVEOUT: *value = c->l1_carveout; return NCG_OK;
    case NCG_TUNE_HULL_STAGE_MIN: *value = c->hstage_min; return NCG_OK;
    case NCG_TUNE_HULL_STAGE_CAP: *value = c->hstage_cap; return NCG_OK;
    case NCG_TUNE_HULL_EPA_WARP: *value = c->hull_epa_warp; return NCG_OK;
    case NCG_TUNE_HULL_LOCALITY: *value = c->hull_locality; return NCG_OK;
    default: g_last_error = "unknown tuning key"; return NCG_EINVAL;
    }
}

int ncg_autotune(ncg_ctx* c, const ncg_batch* b, int query, float param, int reps, int* out_values, float* out_ms,
                 void* stream) {
    if (!c || !b) { g_last_error = "null context or batch"; return NCG_EINVAL; }
    if (query < NCG_QUERY_CONTACT || query > NCG_QUERY_CLOSEST_POINTS) { g_last_error = "unknown query"; return NCG_EINVAL; }
    if (reps < 1 || reps > 64) { g_last_error = "reps must be 1..64"; return NCG_EINVAL; }
    if (query == NCG_QUERY_PROXIMITY && !(param >= 0.0f)) {
        g_last_error = "The proximity margin must be positive or zero.";
        return NCG_EINVAL;
    }
    if (b->n_pairs == 0) { g_last_error = "empty batch"; return NCG_EINVAL; }
    if (!cuda_ok(cudaSetDevice(c->device), "cudaSetDevice")) return NCG_ECUDA;
    cudaStream_t st = (cudaStream_t)stream;
    TuneOutputs t;
    int rc = tune_alloc(query, b->n_pairs, t);
    if (rc != NCG_OK) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int saved_profiling = c->profiling;
    c->profiling = 0;
    auto done = [&](int code) {
        c->profiling = saved_profiling;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(t.buf);
        return code;
    };
    if (!cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&e1), "cudaEventCreate"))
        return done(NCG_ECUDA);
    // candidate values per key, in the order the descent visits the keys
    struct Cand { int key; std::vector<int> values; };
    std::vector<Cand> space = {
        {NCG_TUNE_HULL_GJK_WARP, {0, 1, 8, 9, 10, 11}},
        {NCG_TUNE_HULL_EPA_WARP, {0, 7, 8, 9, 10}},
        {NCG_TUNE_HULL_LOCALITY, {1, 0}},
        {NCG_TUNE_HULL_STAGE_MIN, {0, 1, 64, 256, 512}},
        {NCG_TUNE_HULL_STAGE_CAP, {1024, 2048}},
        {NCG_TUNE_GJK_BLOCKS, {0, 1, 2, 3}},
        {NCG_TUNE_EPA_BLOCKS, {0, 1, 2, 3}},
        {NCG_TUNE_L1_CARVEOUT, {0, -1}},
    };
    int cur[NCG_N_TUNE];
    for (int k = 0; k < NCG_N_TUNE; ++k) ncg_ctx_get_tuning(c, k, &cur[k]);
    float best_ms = 0.0f;
    unsigned long long ref = 0;
    rc = tune_time(c, b, query, param, reps, t, st, e0, e1, &best_ms, &ref);
    if (rc != NCG_OK) return done(rc);
    for (int pass = 0; pass < 2; ++pass) {
        bool changed = false;
        for (const Cand& cd : space) {
            // the stage keys only matter with warp-per-pair hull GJK, the
            // stage size only with staging on
            if (cd.key == NCG_TUNE_HULL_STAGE_MIN && cur[NCG_TUNE_HULL_GJK_WARP] == 0) continue;
            if (cd.key == NCG_TUNE_HULL_STAGE_CAP &&
                (cur[NCG_TUNE_HULL_GJK_WARP] == 0 || cur[NCG_TUNE_HULL_STAGE_MIN] == 0))
                continue;
            for (int v : cd.values) {
                if (v == cur[cd.key]) continue;
                if (ncg_ctx_set_tuning(c, cd.key, v) != NCG_OK) continue;  // not valid on this device
                float ms = 0.0f;
                unsigned long long h = 0;
                rc = tune_time(c, b, query, param, reps, t, st, e0, e1, &ms, &h);
                if (rc != NCG_OK) {
                    ncg_ctx_set_tuning(c, cd.key, cur[cd.key]);
                    return done(rc);
                }
                if (h != ref) {
                    ncg_ctx_set_tuning(c, cd.key, cur[cd.key]);
                    g_last_error = "autotune: outputs changed with tuning key " + std::to_string(cd.key) + " = " +
                                   std::to_string(v);
                    return done(NCG_EINTERNAL);
                }
                if (ms < best_ms * 0.99f) {
                    best_ms = ms;
                    cur[cd.key] = v;
                    changed = true;
                }
                ncg_ctx_set_tuning(c, cd.key, cur[cd.key]);
            }
        }
        if (!changed) break;
    }
    for (int k = 0; k < NCG_N_TUNE; ++k) {
        if (ncg_ctx_set_tuning(c, k, cur[k]) != NCG_OK) return done(NCG_EINTERNAL);
        if (out_values) out_values[k] = cur[k];
    }
    if (out_ms) *out_ms = best_ms;
    return done(NCG_OK);
}

}  // extern "C"
