"""Double-precision model of the FP32 scattering service, for its unit test.

The FP32 path solves for the distance of closest approach with the reference's
Newton steps and stopping test (trim.C:192-233) but starts them from a table of
log2(r0 - b) over (log2 eps, b) (mytrim_gb300/csrc/mtg_newton_guess.h) instead of
the reference's guess (trim.C:183-190) for the universal and Moliere potentials
(C-Kr keeps the reference's guess), and evaluates the magic formula
(trim.C:236-271) with v, v1 at the iterate before the last step, as the
reference does.  This module restates that algorithm in numpy so that the test
can pin the FP32 kernel to it at FP32 rounding level.
"""
import numpy as np

# mtg_newton_guess.h
NG_U, NG_B = 64, 64
NG_U0, NG_U1, NG_BMAX = -18.0, np.log2(10.0), 32.0
NG_DU = (NG_U1 - NG_U0) / (NG_U - 1)
NG_DB = NG_BMAX / (NG_B - 1)

# screening weights w, decay constants k and the reference's derivative
# coefficients c (trim.C:197-222; c = k w except for C-Kr, kept as written)
POT = {
    "universal": (np.array([0.18175, 0.50986, 0.28022, 0.028171]), np.array([3.1998, 0.94229, 0.4029, 0.20162]),
                  None),
    "moliere": (np.array([0.35, 0.55, 0.1]), np.array([0.3, 1.2, 6.0]), np.array([0.105, 0.66, 0.6])),
    "ckr": (np.array([0.191, 0.474, 0.335]), np.array([0.279, 0.637, 1.1919]), np.array([0.531865, 0.30181, 0.6437])),
}
# magic-formula constants (trim.C:236-258)
MAGIC = {
    "universal": (0.011615, 0.0071222, 0.99229, 9.3066, 14.813),
    "moliere": (0.009611, 0.005175, 0.6743, 6.314, 10.0),
    "ckr": (0.235809, 0.126000, 1.0144, 6935.0, 83550.0),
}


def _terms(pot, r):
    w, k, c = POT[pot]
    e = w[None, :] * np.exp(-np.outer(r, k))
    cc = k * w if c is None else c
    return e.sum(1), (e / w[None, :] * cc[None, :]).sum(1)


def guess_table(pot):
    """log2(r0 - b) on the table's grid, r0 by bisection on [b, b + 2 / eps]."""
    u = NG_U0 + np.arange(NG_U) * NG_DU
    b = np.arange(NG_B) * NG_DB
    U, B = np.meshgrid(u, b, indexing="ij")
    eps, B = np.exp2(U.ravel()), B.ravel()
    lo, hi = B.copy(), B + 2.0 / eps
    for _ in range(72):
        m = 0.5 * (lo + hi)
        f = B * B / m + _terms(pot, m)[0] / eps - m
        lo, hi = np.where(f > 0, m, lo), np.where(f > 0, hi, m)
    return np.log2(0.5 * (lo + hi) - B).astype(np.float32).reshape(NG_U, NG_B)


def s2(pot, eps, b, table=None, start="table"):
    """sin^2(theta/2) of the FP32 path's algorithm, evaluated in double; with
    start="reference" every solve starts from the reference's guess (the FP64 path's
    iterates)."""
    eps = np.asarray(eps, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    T = (guess_table(pot) if table is None else table).astype(np.float64)
    out = np.empty_like(eps)
    far = eps > 10.0
    w = 2.0 * eps[far] * b[far]
    out[far] = 1.0 / (1.0 + (1.0 + b[far] * (1.0 + b[far])) * w * w)
    e, bb = eps[~far], b[~far]
    fu = (np.log2(e) - NG_U0) / NG_DU
    fb = bb / NG_DB
    # C-Kr keeps the reference's guess everywhere
    inside = (fu >= 0) & (fb < NG_B - 1) & (pot != "ckr") & (start == "table")
    i = np.clip(fu, 0, NG_U - 2).astype(int)
    j = np.clip(fb, 0, NG_B - 2).astype(int)
    a, c = fu - i, fb - j
    lo = T[i, j] + c * (T[i, j + 1] - T[i, j])
    hi = T[i + 1, j] + c * (T[i + 1, j + 1] - T[i + 1, j])
    d_tab = np.exp2(lo + a * (hi - lo))
    # the reference's guess outside the table (trim.C:183-190)
    with np.errstate(divide="ignore", invalid="ignore"):
        rr = -2.7 * np.log(e * bb)
        rr2 = -2.7 * np.log(e * rr)
    r_ref = np.where((rr >= bb) & (rr2 >= bb), rr2, bb)
    r = np.where(inside, bb + d_tab, r_ref)
    act = np.ones(len(e), bool)
    phi = np.zeros_like(e)
    tk = np.zeros_like(e)
    r_eval = r.copy()
    for _ in range(100):
        ph, t = _terms(pot, r)
        fr = bb * bb / r + ph / e - r
        fr1 = -bb * bb / (r * r) - t / e - 1.0
        q = fr / fr1
        phi, tk, r_eval = np.where(act, ph, phi), np.where(act, t, tk), np.where(act, r, r_eval)
        r = np.where(act, r - q, r)
        act &= np.abs(q) > 1e-3 * np.abs(r)
        if not act.any():
            break
    v = phi / r_eval
    v1 = -(v + tk) / r_eval
    m0, m1, m2, m3, m4 = MAGIC[pot]
    roc = -2.0 * (e - v) / v1
    sqe = np.sqrt(e)
    cc = (m0 + sqe) / (m1 + sqe)
    aa = 2.0 * e * (1.0 + m2 / sqe) * bb ** cc
    ff = (np.sqrt(aa * aa + 1.0) - aa) * ((m3 + e) / (m4 + e))
    co = (bb + (r - bb) * aa * ff / (ff + 1.0) + roc) / (r + roc)
    out[~far] = 1.0 - co * co
    return out


def converged_s2(pot, eps, b):
    """The magic formula at the exact root (bisection), v and v1 there: the value the
    Newton iterates approach."""
    eps = np.asarray(eps, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    lo, hi = b.copy(), b + 2.0 / eps
    for _ in range(200):
        m = 0.5 * (lo + hi)
        f = b * b / m + _terms(pot, m)[0] / eps - m
        lo, hi = np.where(f > 0, m, lo), np.where(f > 0, hi, m)
    r = 0.5 * (lo + hi)
    phi, tk = _terms(pot, r)
    v = phi / r
    v1 = -(v + tk) / r
    m0, m1, m2, m3, m4 = MAGIC[pot]
    roc = -2.0 * (eps - v) / v1
    sqe = np.sqrt(eps)
    cc = (m0 + sqe) / (m1 + sqe)
    aa = 2.0 * eps * (1.0 + m2 / sqe) * b ** cc
    ff = (np.sqrt(aa * aa + 1.0) - aa) * ((m3 + eps) / (m4 + eps))
    co = (b + (r - b) * aa * ff / (ff + 1.0) + roc) / (r + roc)
    return 1.0 - co * co
