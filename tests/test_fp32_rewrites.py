"""Algebraic rewrites of the FP32 face kernel, checked in FP64 against the reference's own
formulas on seeded random cases (CPU, numpy):

* the GIZMO pair limit as one clamp per side (phd_f32.cu gizmo_pair32) against the
  reference's ordered cases, reconstruction.pyx:877-915 -- including the rare
  sign-changing bounds and equal cells;
* the two-rarefaction pressure estimate in closed form against the reference's
  u*-then-average form (riemann.pyx get_waves, the TRRS branch);
* the two-shock estimate's g_K = sqrt(A_K / (p + B_K)) as sqrt(2/(g+1)) / sqrt(d_K (p + B_K)).

The kernel's FP32 arithmetic is checked on the GPU against the FP64 path (L1 density
error, conservation: tests/test_gpu_fp32.py); this file pins the algebra itself."""
import numpy as np

N = 200_000
TOL = 1e-14


def reference_gizmo(sl, sr, ci, cj, xl, xr, qi, qj):
    """reconstruction.pyx:877-915 for one field, vectorised."""
    d1 = 0.5 * np.abs(sl - sr)
    d2 = 0.25 * np.abs(sl - sr)
    mn, mx = np.fmin(sl, sr), np.fmax(sl, sr)
    pbl = sl + qi * (sr - sl)
    pbr = sr + qj * (sl - sr)
    with np.errstate(all="ignore"):
        pp = np.where((mx + d1) * mx >= 0, mx + d1, mx / (1 + d1 / np.abs(mx)))
        pm = np.where((mn - d1) * mn >= 0, mn - d1, mn / (1 + d1 / np.abs(mn)))
    a, b = ci < cj, ci > cj
    left = np.where(a, np.fmax(pm, np.fmin(pbl + d2, xl)), np.where(b, np.fmin(pp, np.fmax(pbl - d2, xl)), sl))
    right = np.where(a, np.fmin(pp, np.fmax(pbr - d2, xr)), np.where(b, np.fmax(pm, np.fmin(pbr + d2, xr)), sr))
    return left, right


def clamp_gizmo(sl, sr, xl, xr, qi, qj):
    """gizmo_pair32's form: outer bound s -/+ d/2 (pulled towards zero where it would
    change sign), inner bound s +/- (q + 1/4) d, one clamp per side."""
    d = sr - sl
    ol, orr = sl - 0.5 * d, sr + 0.5 * d
    il, ir = sl + (qi + 0.25) * d, sr - (qj + 0.25) * d
    with np.errstate(all="ignore"):
        a = np.abs(sl)
        ol = np.where(ol * sl < 0, sl * a / (a + 0.5 * np.abs(d)), ol)
        a = np.abs(sr)
        orr = np.where(orr * sr < 0, sr * a / (a + 0.5 * np.abs(d)), orr)
    return (np.fmin(np.fmax(xl, np.fmin(ol, il)), np.fmax(ol, il)),
            np.fmin(np.fmax(xr, np.fmin(orr, ir)), np.fmax(orr, ir)))


def test_gizmo_clamp_form_equals_the_ordered_cases():
    rng = np.random.default_rng(0)
    ci = rng.normal(size=N) * rng.choice([1e-3, 1.0, 10.0], N)
    cj = ci + rng.normal(size=N) * rng.choice([0.0, 1e-3, 1.0], N)   # a third of the pairs equal
    w = rng.normal(size=N) * rng.choice([0.0, 0.5], N)                # the boost: a common shift
    sl, sr = ci - w, cj - w
    spread = np.abs(sr - sl) + 1e-3
    xl = sl + 2 * spread * rng.normal(size=N)
    xr = sr + 2 * spread * rng.normal(size=N)
    qi, qj = rng.uniform(0.2, 0.8, N), rng.uniform(0.2, 0.8, N)
    l0, r0 = reference_gizmo(sl, sr, ci, cj, xl, xr, qi, qj)
    l1, r1 = clamp_gizmo(sl, sr, xl, xr, qi, qj)
    scale = np.abs(sl) + np.abs(sr) + 1e-300
    assert np.max(np.abs(l0 - l1) / scale) <= TOL
    assert np.max(np.abs(r0 - r1) / scale) <= TOL
    mx = np.fmax(sl, sr)
    mn = np.fmin(sl, sr)
    rare = ((mx + 0.5 * np.abs(sl - sr)) * mx < 0) | ((mn - 0.5 * np.abs(sl - sr)) * mn < 0)
    assert rare.sum() > 1000 and (ci == cj).sum() > 1000        # both special cases exercised


def test_two_rarefaction_closed_form():
    rng = np.random.default_rng(1)
    g = rng.choice([1.4, 5.0 / 3.0], N)
    z = (g - 1) / (2 * g)
    dl, dr = rng.uniform(0.1, 2, N), rng.uniform(0.1, 2, N)
    pl, pr = rng.uniform(0.1, 3, N), rng.uniform(0.1, 3, N)
    ul, ur = rng.uniform(-1, 1, N), rng.uniform(-1, 1, N)
    cl, cr = np.sqrt(g * pl / dl), np.sqrt(g * pr / dr)
    plr = (pl / pr) ** z
    u_star = (plr * ul / cl + ur / cr + 2 * (plr - 1) / (g - 1)) / (plr / cl + 1 / cr)
    with np.errstate(all="ignore"):
        ref = (0.5 * pl * (1 + (g - 1) * (ul - u_star) / (2 * cl)) ** (1 / z) +
               0.5 * pr * (1 + (g - 1) * (u_star - ur) / (2 * cr)) ** (1 / z))
        closed = pr * (plr * ((cl + cr) - 0.5 * (g - 1) * (ur - ul)) / (cl + plr * cr)) ** (1 / z)
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(closed), ok)          # vacuum-generating states: NaN in both
    assert np.max(np.abs(ref - closed)[ok] / ref[ok]) <= 1e-13


def test_two_shock_factor():
    rng = np.random.default_rng(2)
    g = rng.choice([1.4, 5.0 / 3.0], N)
    d, p = rng.uniform(0.1, 2, N), rng.uniform(0.1, 3, N)
    ps = rng.uniform(0.1, 3, N)
    b = p * (g - 1) / (g + 1)
    ref = np.sqrt((2 / ((g + 1) * d)) / (ps + b))
    new = np.sqrt(2 / (g + 1)) / np.sqrt(d * (ps + b))
    assert np.max(np.abs(ref - new) / ref) <= TOL
