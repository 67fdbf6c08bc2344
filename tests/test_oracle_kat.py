"""The oracle against the reference's own known answers (tests/golden/reference_kats.json).

These pin the CPU restatement (oracle/ncg_oracle.hpp) before anything is
compared with it.  Inputs are the reference tests' decimal literals, fed in
f64 (the reference's tests infer f64 for float literals).
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_epa3_cuboid_cuboid_exact():
    k = GOLD["epa3"]
    c = (1, tuple(k["shape"]["half_extents"]), None)
    pairs = [(O.pose8(cs["m1_translation"]), c, O.pose8(cs["m2_translation"]), c) for cs in k["cases"]]
    r = O.query_f64(pairs, O.CONTACT, O.F64, param=k["cases"][0]["prediction"])
    for i, cs in enumerate(k["cases"]):
        assert r.tag[i] == 1
        assert r.value[i] == cs["depth"]          # assert_eq! in the reference
        assert list(r.dir[i]) == cs["normal"]


def test_cylinder_cuboid_issue157():
    k = GOLD["cylinder_cuboid"]
    cyl = (4, (k["cylinder"]["half_height"], k["cylinder"]["radius"]), None)
    cub = (1, tuple(k["cuboid"]["half_extents"]), None)
    pair = [(O.pose8(k["cylinder"]["translation"]), cyl, O.pose8(k["cuboid"]["translation"]), cub)]
    for pol in (O.F64, O.F32, O.MIXED):
        d = O.query_f64(pair, O.DISTANCE, pol)
        p = O.query_f64(pair, O.PROXIMITY, pol, param=k["proximity_margin"])
        c = O.query_f64(pair, O.CONTACT, pol, param=k["contact_prediction"])
        assert d.value[0] == k["distance"]
        assert p.tag[0] == k["proximity"]
        assert c.tag[0] == 1


def test_distance_example():
    k = GOLD["distance_example"]
    ball, cub = (0, (k["ball_radius"],), None), (1, tuple(k["cuboid_half_extents"]), None)
    pairs = [(O.pose8(cs["ball_translation"]), ball, O.pose8(), cub) for cs in k["cases"]]
    r = O.query_f64(pairs, O.DISTANCE, O.F64)
    assert r.value[0] == 0.0
    assert abs(r.value[1] - 1.0) <= k["cases"][1]["epsilon"]


def test_proximity_example():
    k = GOLD["proximity_example"]
    ball, cub = (0, (k["ball_radius"],), None), (1, tuple(k["cuboid_half_extents"]), None)
    pairs = [(O.pose8(cs["ball_translation"]), ball, O.pose8(), cub) for cs in k["cases"]]
    for pol in (O.F64, O.F32, O.MIXED):
        r = O.query_f64(pairs, O.PROXIMITY, pol, param=k["margin"])
        assert list(r.tag) == [cs["proximity"] for cs in k["cases"]]


def test_contact_example_query_dispatch():
    k = GOLD["contact_example"]
    ball, cub = (0, (k["ball_radius"],), None), (1, tuple(k["cuboid_half_extents"]), None)
    pairs = [(O.pose8(cs["ball_translation"]), ball, O.pose8(), cub) for cs in k["cases"]]
    for pol in (O.F64, O.F32, O.MIXED):
        r = O.query_f64(pairs, O.CONTACT_QUERY, pol, param=k["prediction"])
        assert r.tag[0] == 1 and r.value[0] > 0
        assert r.tag[1] == 1 and r.value[1] < 0
        assert r.tag[2] == 0


def test_query_dispatch_ball_ball_is_analytic():
    # contact_ball_ball.rs: depth = r1 + r2 - |c2 - c1|, normal along c2 - c1
    ball = (0, (1.0,), None)
    r = O.query_f64([(O.pose8((0, 0, 0)), ball, O.pose8((1.5, 0, 0)), ball)], O.CONTACT_QUERY, O.F64, param=0.0)
    assert r.tag[0] == 1 and r.value[0] == 0.5
    assert list(r.dir[0]) == [1.0, 0.0, 0.0]
    assert list(r.p1[0]) == [1.0, 0.0, 0.0] and list(r.p2[0]) == [0.5, 0.0, 0.0]
    assert r.counters[0, 1] == 0  # no EPA


def test_johnson_simplex_rejects_degenerate_point():
    k = GOLD["johnson_simplex"]
    for pol in (O.F32, O.F64):
        added, proj, dim = O.simplex_kat(k["points"], pol)
        assert list(added) == k["add_point_results"]
        assert dim <= 2


def test_touching_cuboids_no_nan():
    k = GOLD["touching_cuboids"]
    c = (1, tuple(k["half_extents"]), None)
    pair = [(O.pose8(k["m1_translation"]), c, O.pose8(k["m2_translation"]), c)]
    r = O.query_f64(pair, O.CONTACT, O.F32, param=k["prediction"])
    assert np.all(np.isfinite(r.value)) and np.all(np.isfinite(r.dir))


def test_coincident_cubes_equal_keys():
    # Coincident unit cubes (tests/pipeline/contact_pairs.rs:8-85): GJK ends on
    # a segment through the origin, EPA starts from two flat faces pushed with
    # equal keys (epa3.rs:319-320) and the best face keeps zero barycentric
    # coordinates, so the contact has depth 0 — the reference's pipeline test
    # skips `contact.depth == 0.0` for exactly this configuration.  Every
    # precision must agree, and the normal must be an axis.
    c = (1, (1.0, 1.0, 1.0), None)
    outs = [O.query_f64([(O.pose8(), c, O.pose8(), c)], O.CONTACT, pol, param=0.0) for pol in (O.F64, O.F32, O.MIXED)]
    for r in outs:
        assert r.tag[0] == 1
        assert sorted(np.abs(r.dir[0]).tolist()) == [0.0, 0.0, 1.0]
        assert r.value[0] == 0.0
        assert np.all(np.isfinite(r.p1)) and np.all(np.isfinite(r.p2))


def test_margin_negative_is_rejected():
    c = (1, (1.0, 1.0, 1.0), None)
    with pytest.raises(ValueError):
        O.query_f64([(O.pose8(), c, O.pose8((5, 0, 0)), c)], O.PROXIMITY, O.F64, param=-1.0)


def _toi_batch(pairs):
    from ncollide_gb300 import shapes as S
    shp = np.zeros(2 * len(pairs), S.SHAPE_DTYPE)
    m1 = np.zeros((len(pairs), 8), np.float32)
    m2 = np.zeros((len(pairs), 8), np.float32)
    for i, (t1, s1, t2, s2) in enumerate(pairs):
        for j, (t, sh, m) in enumerate(((t1, s1, m1), (t2, s2, m2))):
            shp[2 * i + j]["kind"] = sh[0]
            shp[2 * i + j]["p"] = list(sh[1]) + [0.0] * (4 - len(sh[1]))
            m[i, 3] = 1.0
            m[i, 4:7] = t
    g1 = np.arange(0, 2 * len(pairs), 2, dtype=np.uint32)
    return S.PairBatch(shp, np.zeros((1, 4), np.float32), m1, g1, m2, g1 + 1)


def test_time_of_impact_ball_cuboid():
    k = GOLD["time_of_impact3_ball_cuboid"]
    ball, cub = (0, (k["ball"]["radius"],)), (1, tuple(k["cuboid"]["half_extents"]))
    b = _toi_batch([(cs["ball_translation"], ball, k["cuboid"]["translation"], cub) for cs in k["cases"]])
    v1 = np.array([cs["ball_vel"] for cs in k["cases"]], np.float32)
    v2 = np.array([cs["box_vel"] for cs in k["cases"]], np.float32)
    r = O.toi(b, v1, v2, O.F64, dispatch=1)
    assert r["some"][0] == 1 and r["toi"][0] == 0.0
    want = (np.sqrt(3.0) - 1.0) / np.linalg.norm(v1[1].astype(np.float64) - v2[1])
    assert r["some"][1] == 1 and abs(r["toi"][1] - want) <= np.finfo(np.float64).eps  # relative_eq!
    assert r["some"][2] == 0
    for pol in (O.F32, O.MIXED):
        rp = O.toi(b, v1, v2, pol, dispatch=1)
        assert list(rp["some"]) == [1, 1, 0] and rp["toi"][0] == 0.0


def test_time_of_impact_ball_ball_analytic():
    k = GOLD["ball_ball_toi"]
    ball = (0, (k["radius"],))
    b = _toi_batch([(k["m1_translation"], ball, k["m2_translation"], ball)])
    r = O.toi(b, np.array([k["vel1"]], np.float32), np.array([k["vel2"]], np.float32), O.F64, dispatch=1)
    assert r["some"][0] == 1 and r["toi"][0] == k["toi"]


def test_time_of_impact_still_objects():
    k = GOLD["still_objects_toi"]
    c = (1, tuple(k["half_extents"]))
    b = _toi_batch([(k["m1_translation"], c, k["m2_translation"], c)] * len(k["cases"]))
    v1 = np.array([[0.0, cs["vel1_y"], 0.0] for cs in k["cases"]], np.float32)
    for pol in (O.F32, O.MIXED):
        r = O.toi(b, v1, np.zeros_like(v1), pol, dispatch=1)
        assert [bool(x) for x in r["some"]] == [cs["some"] for cs in k["cases"]]


def _ray_batch(shape_list):
    from ncollide_gb300 import shapes as S
    shp = np.zeros(len(shape_list), S.SHAPE_DTYPE)
    for i, (kind, prm) in enumerate(shape_list):
        shp[i]["kind"] = kind
        shp[i]["p"] = list(prm) + [0.0] * (4 - len(prm))
    m = np.zeros((len(shape_list), 8), np.float32)
    m[:, 3] = 1.0
    g = np.arange(len(shape_list), dtype=np.uint32)
    return S.PairBatch(shp, np.zeros((1, 4), np.float32), m, g, m, g)


def test_solid_ray_cast_example():
    k = GOLD["solid_ray_cast3d"]
    b = _ray_batch([(1, k["half_extents"])])
    for cs in k["cases"]:
        rays = np.array([cs["origin"] + cs["dir"]], np.float32)
        for pol in (O.F32, O.F64, O.MIXED):
            r = O.ray_cast(b, rays, pol, solid=cs["solid"])
            if cs["toi"] is None:
                assert r["hit"][0] == 0
            else:
                assert r["hit"][0] == 1 and abs(r["toi"][0] - cs["toi"]) <= 1e-6 * max(1.0, cs["toi"])
                if cs["toi"] > 0:  # exit through the +y face
                    assert np.allclose(r["normal"][0], [0.0, 1.0, 0.0], atol=1e-6)


def test_ray_cast_support_maps_analytic_answers():
    # unit cuboid, unit ball, capsule (half height 1, radius 0.5) along y
    b = _ray_batch([(1, (1, 1, 1)), (0, (1,)), (2, (1, 0.5)), (1, (1, 1, 1))])
    rays = np.array([[-5, 0, 0, 1, 0, 0], [-5, 0, 0, 2, 0, 0], [0, -5, 0, 0, 1, 0], [-5, 0, 0, 0, 0, 0]], np.float32)
    for pol in (O.F64, O.MIXED):
        r = O.ray_cast(b, rays, pol)
        assert list(r["hit"]) == [1, 1, 1, 0]
        assert np.allclose(r["toi"][:3], [4.0, 2.0, 3.5], atol=1e-6)
        assert np.allclose(r["normal"][0], [-1, 0, 0], atol=1e-6)
        assert np.allclose(r["normal"][1], [-1, 0, 0], atol=1e-6)
        assert np.allclose(r["normal"][2], [0, -1, 0], atol=1e-6)
        r = O.ray_cast(b, rays, pol, max_toi=3.0)
        assert list(r["hit"]) == [0, 1, 0, 0]


def _cuboid_pairs(pairs):
    from ncollide_gb300 import shapes as S
    shp = np.zeros(2 * len(pairs), S.SHAPE_DTYPE)
    m1 = np.zeros((len(pairs), 8), np.float32)
    m2 = np.zeros((len(pairs), 8), np.float32)
    for i, (t1, h1, t2, h2) in enumerate(pairs):
        shp[2 * i]["kind"] = shp[2 * i + 1]["kind"] = 1
        shp[2 * i]["p"] = list(h1) + [0.0]
        shp[2 * i + 1]["p"] = list(h2) + [0.0]
        m1[i, 3] = m2[i, 3] = 1.0
        m1[i, 4:7] = t1
        m2[i, 4:7] = t2
    g = np.arange(0, 2 * len(pairs), 2, dtype=np.uint32)
    return S.PairBatch(shp, np.zeros((1, 4), np.float32), m1, g, m2, g + 1)


def test_cuboid_manifold_analytic():
    """Face-face manifolds of stacked unit cubes (analytic answers: the corners
    of the overlap rectangle at the penetration depth)."""
    b = _cuboid_pairs([((0, 0, 0), (1, 1, 1), (0, 1.9, 0), (1, 1, 1)),
                       ((0, 0, 0), (1, 1, 1), (0.5, 1.9, 0.3), (1, 1, 1)),
                       ((0, 0, 0), (1, 1, 1), (0, 2.05, 0), (1, 1, 1))])
    r = O.query(b, O.CONTACT, O.F32, param=0.1)
    c9 = np.concatenate([r.p1, r.p2, r.dir], 1).astype(np.float32)
    man, st = O.manifold(b, c9, r.tag, linear=0.1, angular1=0.1, angular2=0.1)
    assert not st.any()
    corners = lambda m: {(round(float(p["world1"][0]), 5), round(float(p["world1"][2]), 5))
                         for p in m["points"][:m["n"]]}
    assert man[0]["n"] == 8 and corners(man[0]) == {(1, 1), (1, -1), (-1, 1), (-1, -1)}
    assert man[1]["n"] == 4 and corners(man[1]) == {(1, 1), (1, -0.7), (-0.5, 1), (-0.5, -0.7)}
    for m, d in ((man[0], 0.1), (man[1], 0.1), (man[2], -0.05)):
        pts = m["points"][:m["n"]]
        assert np.allclose(pts["depth"], d, atol=1e-6)
        assert np.allclose(pts["world1"][:, 1], 1.0) and np.allclose(m["normal"], [0, 1, 0], atol=1e-7)
    # features: cube 1's +y face is Face(1), cube 2's -y face Face(4)
    assert {int(p["feature2"]) for p in man[0]["points"][:4]} == {(3 << 28) | 4}
    assert {int(p["feature1"]) for p in man[0]["points"][4:8]} == {(3 << 28) | 1}
