"""The mixed path's near-wing KAPMIN cutoff search (``pair_wings`` in
``csrc/ks_kernels.cuh``) against the reference's offset-by-offset scan
(synthe_py/physics/line_opacity.py:474-537).

The kernel scans offsets one by one only while they map below table index 5,
then searches: it starts at the analytic crossing of
kappa0 * (exp(-v^2) + 0.5642 a / v^2) with KAPMIN, gallops down or up from
there and bisects.  That returns the scan's offset as long as the FP32
profile H0 + a*H1 does not increase from table index 5 on for a < 0.2, which
the first tests check on the tables; the last test runs a restatement of the
kernel's search on FP32 profiles and compares it with the scan.
"""

from pathlib import Path

import numpy as np

TABLES = np.load(Path(__file__).parent / "golden" / "tables_ref.npz")
f32 = np.float32
H0 = TABLES["h0tab"].astype(np.float32)
H1 = TABLES["h1tab"].astype(np.float32)


def test_table_profile_non_increasing_from_index_5():
    # H0 + a*H1 is linear in a: non-increasing for a in [0, 0.2] iff at both ends
    for a in (0.0, 0.2):
        v = H0.astype(np.float64) + a * H1.astype(np.float64)
        assert np.all(np.diff(v[5:]) <= 0.0), a


def test_asymptote_below_last_table_value():
    # beyond v = 10 the profile is 0.5642 a / v^2, below the table's last value
    for a in np.linspace(1e-6, 0.2, 50):
        assert 0.5642 * a / 100.0 <= float(H0[-1]) + a * float(H1[-1])


def _profile(o, dv, ad, k0):
    """near_profile<float> for a < 0.2 (line_opacity.py:474-491)."""
    x = f32(f32(o) * dv)
    if x > f32(10):
        return f32(k0 * f32(f32(f32(0.5642) * ad) / f32(x * x)))
    idx = min(max(int(f32(f32(0.5) + f32(f32(o) * f32(f32(200) * dv)))), 0), 2000)
    return f32(k0 * f32(H0[idx] + f32(ad * H1[idx])))


def _scan(n10, dv, ad, k0, km):
    for o in range(1, n10 + 1):
        if _profile(o, dv, ad, k0) < km:
            return o
    return -1


def _kernel_search(n10, dv, ad, k0, km, start=None):
    """The kernel's order of probes; ``start`` in [0, 1) replaces the analytic
    start by that fraction of the searched range [ns, n10]."""
    ns = 1
    while ns <= n10:
        if int(f32(f32(0.5) + f32(f32(ns) * f32(f32(200) * dv)))) >= 5:
            break
        if _profile(ns, dv, ad, k0) < km:
            return ns
        ns += 1
    if ns > n10:
        return -1
    g = n10
    r = f32(km / k0)
    if 0.0 < r < 1.0:
        v = max(np.sqrt(-np.log(r)), np.sqrt(f32(0.5642) * ad / r))
        og = v / dv
        if og < n10:
            g = max(ns, int(og))
    elif r >= 1.0:
        g = ns
    if start is not None:
        g = ns + min(int(start * (n10 - ns + 1)), n10 - ns)
    lo, hi = ns - 1, -1
    if _profile(g, dv, ad, k0) < km:
        hi, step = g, 1
        while hi - lo > 1:
            probe = max(hi - step, lo + 1)
            if _profile(probe, dv, ad, k0) < km:
                hi, step = probe, step * 2
            else:
                lo = probe
                break
    elif g != n10:
        lo, probe, step = g, g + 1, 1
        while True:
            if _profile(probe, dv, ad, k0) < km:
                hi = probe
                break
            lo = probe
            if probe == n10:
                break
            probe, step = min(probe + step, n10), step * 2
    if hi < 0:
        return -1
    while hi - lo > 1:
        mid = lo + ((hi - lo) >> 1)
        if _profile(mid, dv, ad, k0) < km:
            hi = mid
        else:
            lo = mid
    return hi


def test_search_matches_scan_on_fp32_profiles():
    rng = np.random.default_rng(7)
    for _ in range(3000):
        dv = f32(10 ** rng.uniform(-2.5, 0.3))
        ad = f32(rng.uniform(0, 0.2) if rng.random() < 0.8 else 10 ** rng.uniform(-6, -0.7))
        k0 = f32(10 ** rng.uniform(-5, 5))
        n10 = int(rng.integers(1, 120))
        ref = int(rng.integers(1, n10 + 1))
        km = f32(_profile(ref, dv, ad, k0) * f32(10 ** rng.uniform(-0.01, 0.01)))
        u = rng.random()
        if u < 0.2:
            km = _profile(ref, dv, ad, k0)  # exact tie with a profile value
        elif u < 0.25:
            km = f32(k0 * 2)  # above the whole profile: cut at the first offset
        elif u < 0.3:
            km = f32(0)  # never crossed
        want = _scan(n10, dv, ad, k0, km)
        assert _kernel_search(n10, dv, ad, k0, km) == want
        assert _kernel_search(n10, dv, ad, k0, km, start=rng.random()) == want
