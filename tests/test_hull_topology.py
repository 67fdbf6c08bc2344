"""ConvexHull face topology (ncg_hull_topology_build: the hull's triangles,
then ConvexHull::try_new, src/shape/convex.rs:88-328) on the CPU: known
polyhedra, the invariants try_new establishes, degenerate inputs, and the
oracle's manifold of a Cuboid given as a ConvexHull of its corners against
the Cuboid's own."""
import itertools

import numpy as np

from ncollide_gb300 import hulls as H
from ncollide_gb300 import shapes as S
from ncollide_gb300 import workloads as W
from oracle import oracle as O


def topo_of(point_sets):
    pairs = [(S.isometry(), S.ConvexHull(np.asarray(p, np.float32)), S.isometry(), S.Ball(1.0)) for p in point_sets]
    b = S.pack_pairs(pairs)
    return b, H.HostTopology(b)


def hull_ids(b):
    return np.nonzero(b.shapes["kind"] == S.CONVEX_HULL)[0]


def test_cube_corners_give_six_square_faces():
    corners = np.array(list(itertools.product((-0.5, 0.5), repeat=3)), np.float32) * np.array([1.0, 0.6, 0.3], np.float32)
    b, T = topo_of([corners])
    s = hull_ids(b)[0]
    f0, nf, e0, ne = T.arrays["shape"][s]
    assert nf == 6 and T.n_failed == 0
    fr = T.arrays["face_range"][f0:f0 + nf]
    assert (fr[:, 1] == 4).all()                      # the two triangles of each side merged
    n = T.arrays["face_normal"][f0:f0 + nf, :3]
    assert sorted(map(tuple, np.rint(n).astype(int))) == sorted(
        [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)])
    # 12 kept edges plus the 6 deleted diagonals; V - E + F = 2 over kept edges
    assert ne == 18
    used = np.unique(T.arrays["face_edge"][fr[0, 0]:fr[-1, 0] + fr[-1, 1]])
    assert len(used) == 12 and 8 - 12 + 6 == 2


def test_tetrahedron_and_degenerate_sets():
    tet = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]]
    flat = [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0.5, 0.5, 0]]
    line = [[0, 0, 0], [1, 1, 1], [2, 2, 2], [3, 3, 3]]
    b, T = topo_of([tet, flat, line])
    ids = hull_ids(b)
    assert T.arrays["shape"][ids[0], 1] == 4
    assert T.arrays["shape"][ids[1], 1] == 0 and T.arrays["shape"][ids[2], 1] == 0
    assert T.n_failed == 2


def test_random_hulls_satisfy_try_new_invariants():
    b = W.hull_pairs_pooled(64, seed=3, pool=256, kinds=(S.CONVEX_HULL,))
    T = H.HostTopology(b)
    pts = b.hull_points[:, :3].astype(np.float64)
    ok = 0
    for s in hull_ids(b):
        f0, nf, e0, ne = (int(x) for x in T.arrays["shape"][s])
        if nf == 0:
            continue
        ok += 1
        off, cnt = int(b.shapes["hull_off"][s]), int(b.shapes["hull_n"][s])
        P = pts[off:off + cnt]
        centre = P.mean(0)
        fr = T.arrays["face_range"][f0:f0 + nf]
        normals = T.arrays["face_normal"][f0:f0 + nf, :3].astype(np.float64)
        assert np.allclose(np.linalg.norm(normals, axis=1), 1.0, atol=1e-5)
        deg = np.zeros(cnt, int)
        for (first, count), nrm in zip(fr, normals):
            vid = T.arrays["face_vertex"][first:first + count]
            np.add.at(deg, vid, 1)
            fc = P[vid].mean(0)
            assert np.dot(nrm, fc - centre) > 0.0                       # outward
            assert (P @ nrm - np.dot(P[vid[0]], nrm)).max() < 2e-2     # every point behind the face
        vr = T.arrays["vertex_range"][off:off + cnt]
        assert np.array_equal(vr[:, 1], deg)                            # faces around each vertex
        kept = np.unique(np.concatenate([T.arrays["face_edge"][a:a + c] for a, c in fr]))
        assert (deg > 0).sum() - len(kept) + nf == 2                    # Euler characteristic
    assert ok > 200


def test_oracle_cube_hull_manifold_equals_cuboid_manifold():
    """Resting cuboids and the same cuboids given as ConvexHulls of their eight
    corners: the same contact points and depths (feature ids are each shape's own)."""
    base = W.cuboid_stacks(256, seed=5)
    corners = np.array(list(itertools.product((-1.0, 1.0), repeat=3)))
    pairs_c, pairs_h = [], []
    for i in range(base.n_pairs):
        h1, h2 = base.shapes["p"][base.g1[i], :3], base.shapes["p"][base.g2[i], :3]
        m1 = (base.m1[i, 4:7], base.m1[i, :4])
        m2 = (base.m2[i, 4:7], base.m2[i, :4])
        pairs_c.append((S.isometry(*m1), S.Cuboid(h1), S.isometry(*m2), S.Cuboid(h2)))
        pairs_h.append((S.isometry(*m1), S.ConvexHull((corners * h1).astype(np.float32)), S.isometry(*m2),
                        S.ConvexHull((corners * h2).astype(np.float32))))
    bc, bh = S.pack_pairs(pairs_c), S.pack_pairs(pairs_h)
    T = H.HostTopology(bh)
    assert T.n_failed == 0
    rc = O.query(bc, O.CONTACT, O.MIXED, param=0.1, eps=-1.0, epa_tol=1e-6)
    c9 = np.concatenate([rc.p1, rc.p2, rc.dir], 1).astype(np.float32)
    mc, sc = O.manifold(bc, c9, rc.tag, linear=0.1, angular1=0.05, angular2=0.05)
    mh, sh = O.manifold(bh, c9, rc.tag, linear=0.1, angular1=0.05, angular2=0.05, topology=T)
    assert not (sh & 0x200).any() and not (sc & 0x200).any()
    assert np.array_equal(mc["n"], mh["n"])
    agree = 0
    for i in np.nonzero(rc.tag == 1)[0]:
        k = mc["n"][i]
        a = np.sort(np.concatenate([mc["points"]["world1"][i, :k], mc["points"]["depth"][i, :k, None]], 1), 0)
        h = np.sort(np.concatenate([mh["points"]["world1"][i, :k], mh["points"]["depth"][i, :k, None]], 1), 0)
        agree += np.allclose(a, h, atol=1e-5)
    assert agree >= 0.95 * (rc.tag == 1).sum()
