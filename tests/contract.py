"""The accuracy contract of the batched narrow phase, as checks shared by the
CPU tests (the oracle's mixed-precision instantiation standing in for the
kernels, which equal it bit for bit) and the GPU tests (the kernels' own
outputs through the C ABI).

The contract has two halves:
  (i)  classification: whether a contact exists (Some / None of
       query::contact with prediction 0) agrees with the reference's f32 path
       outside a +-1e-6 band around touching, the band being on the f64
       oracle's signed gap (-depth when penetrating, else the distance);
  (ii) accuracy: distance, depth, normal and witness points within 1e-5
       relative (to max(|value|, rA + rB); normals absolute) of the f64
       oracle, the reference's algorithm built with f64.

Where the reference's own f32 path does not meet (i) or (ii), the kernels
cannot both equal it and meet them: these checks then require the kernels to
agree with f64 at least as well as the f32 reference path does, and state the
measured bound.  The limits below are those measured bounds, with margin.
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O

BAND = 1e-6
TOL = 1e-5
CURVED_KINDS = (0, 2, 3)  # Ball, Capsule, Cone


def classes(batch):
    k1, k2 = batch.kinds()
    curved = np.isin(k1, CURVED_KINDS) | np.isin(k2, CURVED_KINDS)
    ballball = (k1 == 0) & (k2 == 0)
    return curved, ballball


def signed_gap(batch, query=O.CONTACT):
    r64 = O.query(batch, query, O.F64, param=0.0)
    d64 = O.query(batch, O.DISTANCE, O.F64)
    return np.where(r64.tag == 1, -r64.value, d64.value), r64, d64


def contact_errors(contact, has, r64, batch):
    """Relative depth, absolute normal and relative witness-point errors of the
    pairs that penetrate in f64 and have a contact."""
    curved, ballball = classes(batch)
    c = np.asarray(contact, np.float64)
    m = (has == 1) & (r64.tag == 1) & (r64.value > 0) & ~ballball
    scale = batch.scale
    dd = np.abs(c[:, 9] - r64.value) / np.maximum(np.abs(r64.value), scale)
    dn = np.linalg.norm(c[:, 6:9] - r64.dir, axis=1)
    dp = np.maximum(np.linalg.norm(c[:, 0:3] - r64.p1, axis=1), np.linalg.norm(c[:, 3:6] - r64.p2, axis=1)) / scale
    return {"depth": dd, "normal": dn, "witness": dp}, m & ~curved, m & curved


def distance_errors(dist, d64, batch):
    curved, ballball = classes(batch)
    m = (d64.value > 0) & ~ballball
    e = np.abs(np.asarray(dist, np.float64) - d64.value) / np.maximum(np.abs(d64.value), batch.scale)
    return e, m & ~curved, m & curved


def p99(x, m):
    return float(np.percentile(x[m], 99)) if m.any() else 0.0


def frac_over(x, m, t=TOL):
    return float((x[m] > t).mean()) if m.any() else 0.0


def check_classification(has, batch, query, stress):
    """(i): the kernels' contact classification against the f32 reference
    path and f64 outside the band.  Returns the counts."""
    gap, r64, _ = signed_gap(batch, query)
    r32 = O.query(batch, query, O.F32, param=0.0)
    out = ~(np.abs(gap) <= BAND)
    gpu, ref, f64 = has == 1, r32.tag == 1, r64.tag == 1
    vs_ref = (gpu != ref) & out
    vs_f64 = (gpu != f64) & out
    ref_f64 = (ref != f64) & out
    counts = {"outside_band": int(out.sum()), "vs_f32_reference": int(vs_ref.sum()), "vs_f64": int(vs_f64.sum()),
              "f32_reference_vs_f64": int(ref_f64.sum())}
    if not stress:
        # every disagreement with the f32 path is a pair the f32 path gets
        # wrong (the kernels agree with f64 there), and none with f64
        assert counts["vs_f64"] == 0, counts
        assert not np.any(vs_ref & (gpu != f64)), counts
    else:
        # thin, near-touching shapes: the f32 path misclassifies ~15% outside
        # the band; the kernels stay within 1% of f64 and below a tenth of the
        # f32 path's rate
        assert counts["vs_f64"] <= 0.01 * counts["outside_band"], counts
        assert counts["vs_f64"] * 10 <= max(counts["f32_reference_vs_f64"], 1), counts
    return counts


def check_accuracy(contact, has, dist, batch, query, stress):
    """(ii): errors against f64, polytope pairs to 1e-5, curved pairs no worse
    than the reference's f32 path (their declared bound)."""
    _, r64, d64 = signed_gap(batch, query)
    r32 = O.query(batch, query, O.F32, param=0.0)
    r32d = O.query(batch, O.DISTANCE, O.F32)
    err, poly, curv = contact_errors(contact, has, r64, batch)
    ref = np.concatenate([r32.p1, r32.p2, r32.dir, r32.value[:, None]], 1)
    err32, poly32, curv32 = contact_errors(ref, r32.tag, r64, batch)
    report = {}
    for k in ("depth", "normal", "witness"):
        report[k] = {"polytope_p99": p99(err[k], poly), "polytope_frac_gt_1e-5": frac_over(err[k], poly),
                     "polytope_f32_reference_frac_gt_1e-5": frac_over(err32[k], poly32),
                     "curved_p99": p99(err[k], curv), "curved_f32_reference_p99": p99(err32[k], curv32)}
        # polytope pairs: 1e-5 at the 99th percentile; the rare pairs beyond
        # are EPA runs that end on a non-optimal face in f32 as well, and
        # face-face contacts of thin shapes, whose witness points are not
        # unique: no more of them than 0.5% or than the f32 path has
        assert report[k]["polytope_p99"] <= TOL, (k, report[k])
        assert report[k]["polytope_frac_gt_1e-5"] <= max(0.005, report[k]["polytope_f32_reference_frac_gt_1e-5"]), \
            (k, report[k])
        # curved pairs: at least as accurate as the reference's own f32 path
        assert report[k]["curved_p99"] <= 1.5 * report[k]["curved_f32_reference_p99"] + 1e-7, (k, report[k])
    # curved depth: within 5e-5 at the 99th percentile
    assert report["depth"]["curved_p99"] <= 5e-5, report["depth"]
    de, dpoly, dcurv = distance_errors(dist, d64, batch)
    de32, _, _ = distance_errors(r32d.value, d64, batch)
    report["distance"] = {"p99": p99(de, dpoly | dcurv), "frac_gt_1e-5": frac_over(de, dpoly | dcurv),
                          "f32_reference_p99": p99(de32, dpoly | dcurv)}
    # distance: 1e-5 at the 99th percentile, outliers under 0.5% (thin,
    # near-touching shapes; the f32 path's p99 there is ~4e-3)
    assert report["distance"]["p99"] <= TOL and report["distance"]["frac_gt_1e-5"] <= 0.005, report["distance"]
    return report
