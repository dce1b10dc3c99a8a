"""Parity checks of traced hits against the oracle (shared by the GPU tests)."""
import numpy as np

from visionaray_gb300.types import NO_HIT


def ulp_diff(a, b):
    """Distance in float32 ulps (sign-aware, via the ordered-int mapping)."""
    ai = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    bi = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    ai = np.where(ai < 0, -(ai & 0x7FFFFFFF), ai)
    bi = np.where(bi < 0, -(bi & 0x7FFFFFFF), bi)
    return np.abs(ai - bi)


def compare_closest(got, ref, rays, tris_by_prim, oracle, max_t_ulp=2):
    """Closest-hit parity: prim_id must equal the oracle's except for equal-t ties
    (another triangle hit within `max_t_ulp` of the oracle's t, re-verified with the
    oracle's own ray/triangle test); where prim_id agrees, t, u, v are compared in
    ulps.  Returns a stats dict; raises AssertionError on any unexplained mismatch."""
    gp, rp = got["prim_id"], ref["prim_id"]
    same = gp == rp
    stats = {"rays": int(len(rays)), "hits": int((rp != NO_HIT).sum()), "prim_mismatch": int((~same).sum())}
    bad = []
    ties = 0
    for i in np.nonzero(~same)[0]:
        if gp[i] == NO_HIT or rp[i] == NO_HIT:
            bad.append((int(i), "hit/miss disagreement", int(gp[i]), int(rp[i])))
            continue
        hit, rec = oracle.intersect(rays[i], tris_by_prim[gp[i]])
        if not hit or rec["t"] != got["t"][i]:
            bad.append((int(i), "reported hit not reproduced by the oracle", int(gp[i]), int(rp[i])))
            continue
        if ulp_diff(got["t"][i], ref["t"][i]) > max_t_ulp:
            bad.append((int(i), "different triangle at a different t", float(got["t"][i]), float(ref["t"][i])))
            continue
        ties += 1
    stats["ties"] = ties
    hit = same & (rp != NO_HIT)
    for f in ("t", "u", "v"):
        d = ulp_diff(got[f][hit], ref[f][hit]) if hit.any() else np.zeros(1, np.int64)
        stats[f"max_ulp_{f}"] = int(d.max()) if d.size else 0
        stats[f"exact_{f}"] = float((d == 0).mean()) if d.size else 1.0
    assert not bad, f"{len(bad)} unexplained mismatches, first: {bad[:5]}"
    for f in ("t", "u", "v"):
        assert stats[f"max_ulp_{f}"] <= max_t_ulp, stats
    return stats


def compare_any(got, ref, rays, tris_by_prim, oracle):
    """Any-hit parity: the occlusion flag must equal the oracle's for every ray, and
    each reported hit must be a real hit inside [tmin, tmax] (which triangle is
    reported depends on traversal order, as in the reference)."""
    g_occ = got["prim_id"] != NO_HIT
    r_occ = ref["prim_id"] != NO_HIT
    mism = np.nonzero(g_occ != r_occ)[0]
    assert len(mism) == 0, f"{len(mism)} occlusion mismatches, first {mism[:10]}"
    idx = np.nonzero(g_occ)[0]
    step = max(1, len(idx) // 2000)
    for i in idx[::step]:
        hit, rec = oracle.intersect(rays[i], tris_by_prim[got["prim_id"][i]])
        assert hit and rec["t"] == got["t"][i], i
        assert rays["tmin"][i] <= got["t"][i] <= rays["tmax"][i], i
    return {"rays": int(len(rays)), "occluded": int(g_occ.sum())}


def non_finite_soup(n_good=20000, seed=9):
    """A triangle soup with 20 zero-area, 20 NaN-vertex and 20 Inf-vertex triangles
    inserted after the first half (prim ids = positions; the bad ones are
    n_good // 2 .. n_good // 2 + 59)."""
    from visionaray_gb300 import scenes
    good = scenes.soup(n_good, seed=seed)
    bad = np.zeros(60, good.dtype)
    rng = np.random.default_rng(2)
    bad["v1"] = rng.uniform(0, 1, size=(60, 3))
    bad["e1"][:20] = (0.1, 0.0, 0.0)   # zero area: e2 parallel to e1
    bad["e2"][:20] = (0.2, 0.0, 0.0)
    bad["v1"][20:40, 1] = np.nan
    bad["e1"][20:40] = (0.05, 0.0, 0.0)
    bad["e2"][20:40] = (0.0, 0.05, 0.0)
    bad["v1"][40:] = (np.inf, 0.5, 0.5)
    bad["e1"][40:] = (0.05, 0.0, 0.0)
    bad["e2"][40:] = (0.0, 0.05, 0.0)
    h = n_good // 2
    tris = np.concatenate([good[:h], bad, good[h:]])
    tris["prim_id"] = np.arange(len(tris))
    tris["geom_id"] = 0
    return tris
