"""Per-family parity rules shared by the oracle tests and the GPU tests.

Feature families are identified by the group name of each feature.  Three
kinds of comparison:
  * "float": |a-b| <= rtol*|b| + atol;
  * "counts": histogram-like groups whose values come from binning a
    floating-point quantity: they may differ by a few single-count moves
    between neighbouring bins (each move changes two entries by 1); the
    number of such moves per group is budgeted;
  * "f14": Haralick maximal-correlation-coefficient entries (in-group
    indices 16, 17): sqrt of eigenvalue #2 in Schur order, which depends on
    the eigen-solver's rounding (two builds of the reference itself differ);
    reported, never gated beyond "finite and in [0, 1.5]".
"""
import numpy as np

F14 = (16, 17)
COUNT_GROUPS = ("Chebyshev-Fourier Coefficients", "Chebyshev Coefficients", "Comb Moments",
                "Radon Coefficients", "Multiscale Histograms")


def group_of(name):
    return name.rsplit(" [", 1)[0]


def index_of(name):
    return int(name.rsplit("[", 1)[1].rstrip("]"))


def compare(a, b, names, rtol=1e-6, atol=1e-9, count_moves=2, skip=()):
    """Compare feature rows a (candidate) and b (expected).  Returns a dict of
    failures keyed by group name; empty when everything is within rules."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    groups = {}
    for i, n in enumerate(names):
        groups.setdefault(group_of(n), []).append(i)
    fails = {}
    for g, idx in groups.items():
        if any(g.startswith(s) for s in skip):
            continue
        idx = np.array(idx)
        alg = g.split(" (")[0]
        va, vb = a[idx], b[idx]
        if alg == "Haralick Textures":
            f14 = np.array([index_of(names[i]) in F14 for i in idx])
            bad14 = ~np.isfinite(va[f14]) | (va[f14] < 0) | (va[f14] > 1.5)
            if bad14.any():
                fails[g] = ("f14 out of range", va[f14])
            va, vb = va[~f14], vb[~f14]
        if alg in COUNT_GROUPS:
            d = np.abs(va - vb)
            if alg == "Multiscale Histograms":
                ok = np.allclose(va, vb, rtol=rtol, atol=0.02)
            else:
                ok = (np.abs(np.round(d) - d) < 1e-9).all() and d.sum() <= 2 * count_moves
            if not ok:
                fails[g] = ("counts", d.sum(), np.nonzero(d)[0][:8])
            continue
        tol = rtol * np.abs(vb) + atol
        bad = np.abs(va - vb) > tol
        if bad.any():
            j = np.nonzero(bad)[0]
            fails[g] = ("float", j[:8].tolist(), va[j[:4]].tolist(), vb[j[:4]].tolist())
    return fails


# Mixed-precision form: families whose kernels compute in FP32 carry their own
# stated tolerance; every other family keeps the FP64 rules above.
#   ("float", rtol, gtol): |a-b| <= rtol*|b| + gtol*max|group|
#   ("counts", moves):     at most `moves` single-count moves per group
MIXED_RULES = {
    "Chebyshev-Fourier Coefficients": ("counts", 3),
    # ratios of threshold counts over FP32 filter energies: a few pixels of the
    # 512 x 512 maps may cross the threshold
    "Gabor Textures": ("float", 1e-4, 0.0),
}


def compare_mixed(a, b, names, rtol=1e-7, atol=1e-9, count_moves=2, skip=()):
    """compare() with the mixed form's per-family tolerances."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    fails = compare(a, b, names, rtol, atol, count_moves, skip=tuple(skip) + tuple(MIXED_RULES))
    groups = {}
    for i, n in enumerate(names):
        groups.setdefault(group_of(n), []).append(i)
    for g, idx in groups.items():
        alg = g.split(" (")[0]
        if alg not in MIXED_RULES or any(g.startswith(s) for s in skip):
            continue
        rule = MIXED_RULES[alg]
        va, vb = a[idx], b[idx]
        if rule[0] == "counts":
            d = np.abs(va - vb)
            if not ((np.abs(np.round(d) - d) < 1e-9).all() and d.sum() <= 2 * rule[1]):
                fails[g] = ("counts", d.sum(), np.nonzero(d)[0][:8])
        else:
            scale = np.max(np.abs(vb)) if len(vb) else 0.0
            bad = np.abs(va - vb) > rule[1] * np.abs(vb) + rule[2] * scale
            if bad.any():
                j = np.nonzero(bad)[0]
                fails[g] = ("float", j[:8].tolist(), va[j[:4]].tolist(), vb[j[:4]].tolist())
    return fails


def family_errors(a, b, names):
    """Per family (algorithm name): max |a-b| / max(|b|, 1e-300) over entries
    and max |a-b| / max|group|, for reporting."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    out = {}
    groups = {}
    for i, n in enumerate(names):
        groups.setdefault(group_of(n), []).append(i)
    for g, idx in groups.items():
        alg = g.split(" (")[0]
        va, vb = a[idx], b[idx]
        if alg == "Haralick Textures":
            keep = np.array([index_of(names[i]) not in F14 for i in idx])
            va, vb = va[keep], vb[keep]
        fin = np.isfinite(va) & np.isfinite(vb)
        va, vb = va[fin], vb[fin]
        if not len(va):
            continue
        d = np.abs(va - vb)
        relv = d / np.maximum(np.abs(vb), 1e-300)
        rel = float(np.max(relv))
        grel = float(np.max(d) / max(np.max(np.abs(vb)), 1e-300))
        r0, g0, w0 = out.get(alg, (0.0, 0.0, ""))
        if grel > g0:
            k = int(np.argmax(d))
            w0 = "%s (%.6g vs %.6g)" % (g, va[k], vb[k])
        out[alg] = (max(r0, rel), max(g0, grel), w0)
    return out
