"""TEST INFRASTRUCTURE: a float64 torch restatement of the differentiable
part of the path, for checking the hand-written backward kernels against
torch autograd.  Each function restates the reference computation it names
(the same formulas as oracle/wc_oracle.cpp; torch only adds the derivative):

  fourier    ImageMatrix::fft2 (src/cmatrix.cpp:1107-1200): |DFT2|
  chebyshev  Chebyshev2D (src/transforms/chebyshev.cpp:39-165): A^T x^T B
  wavelet    one level of Symlet-5, zero-padded (Wavelet.cpp:136-434)
  edge       EdgeTransform (src/cmatrix.cpp:1294-1311), std::max's tie order
  zernike    mb_zernike2D (src/textures/zernike/zernike.cpp:207-341)
  pixstats   PixelIntensityStatistics (src/FeatureAlgorithms.cpp:272-294)
  fractal    FractalFeatures (src/FeatureAlgorithms.cpp:232-267)
  gini       GiniCoefficient (src/FeatureAlgorithms.cpp:448-492)
  wnd        signatures::normalize + classify2 (TrainingSet.cpp:2429-2586)
"""
import math

import numpy as np
import torch

EPS = np.finfo(np.float64).eps
SYM_LO = [0.027333068345077982, 0.029519490925774643, -0.039134249302383094, 0.1993975339773936,
          0.72340769040242059, 0.63397896345821192, 0.016602105764522319, -0.17532808990845047,
          -0.021101834024758855, 0.019538882735286728]
SYM_HI = [-0.019538882735286728, -0.021101834024758855, 0.17532808990845047, 0.016602105764522319,
          -0.63397896345821192, 0.72340769040242059, -0.1993975339773936, -0.039134249302383094,
          -0.029519490925774643, 0.027333068345077982]


def fourier(x):
    return torch.fft.fft2(x).abs()


def cheb_factor(length, N):
    A = np.zeros((length, N))
    for a in range(length):
        xx = 2 * (a + 1) / length - 1
        ac = 0.0 if abs(xx) > 1 else math.acos(xx)
        for j in range(N):
            t = 1.0 if j == 0 else math.cos(ac * j)
            t = t / length if j == 0 else t * 2 / length
            A[a, j] = t / 2
    return torch.from_numpy(A)


def chebyshev(x):
    H, W = x.shape
    N = min(W, H)
    A, B = cheb_factor(W, N), cheb_factor(H, N)
    oh = min(H, N)
    return (A.T @ (x.T @ B))[:oh]


def _dec(n, taps):
    o = (n + 9) // 2
    M = np.zeros((o, n))
    for r in range(o):
        for j in range(10):
            k = 2 * r + 1 - j
            if 0 <= k < n:
                M[r, k] = taps[j]
    return torch.from_numpy(M)


def wavelet(x):
    Y, X = x.shape
    ta, td = _dec(Y, SYM_LO) @ x, _dec(Y, SYM_HI) @ x
    LoX, HiX = _dec(X, SYM_LO), _dec(X, SYM_HI)
    a1, d1, a2, d2 = ta @ LoX.T, ta @ HiX.T, td @ LoX.T, td @ HiX.T
    return torch.cat([torch.cat([d2, d1], 1), torch.cat([a2, a1], 1)], 0)


def _pick(a, b):
    # std::max(a, b): b when a < b, else a
    return torch.where(a < b, b, a)


def edge(x):
    H, W = x.shape
    myy = torch.zeros_like(x)
    mxx = torch.zeros_like(x)
    if H > 2:
        c = x[1:-1]
        myy = torch.cat([x[:1] * 0, _pick((c - x[:-2]).abs(), (c - x[2:]).abs()), x[:1] * 0], 0)
    if W > 2:
        c = x[:, 1:-1]
        mxx = torch.cat([x[:, :1] * 0, _pick((c - x[:, :-2]).abs(), (c - x[:, 2:]).abs()), x[:, :1] * 0], 1)
    return _pick(mxx, myy)


TRANSFORMS = {"Fourier": fourier, "Chebyshev": chebyshev, "Wavelet": wavelet, "Edge": edge}


def chain_of(group_chain_text):
    """'(Chebyshev (Fourier ()))' -> ['Fourier', 'Chebyshev'] (application order)."""
    names = [t for t in group_chain_text.replace("(", " ").replace(")", " ").split() if t]
    return names[::-1]


def _zernike_coeffs():
    H1, H2, H3 = np.zeros((16, 16)), np.zeros((16, 16)), np.zeros((16, 16))
    for n in range(16):
        for m in range(n + 1):
            if n != m:
                H3[n, m] = -(4.0 * (m + 2.0) * (m + 1.0)) / ((n + m + 2.0) * (n - m))
                H2[n, m] = (H3[n, m] * (n + m + 4.0) * (n - m - 2.0)) / (4.0 * (m + 3.0)) + (m + 2.0)
                H1[n, m] = ((m + 4.0) * (m + 3.0)) / 2.0 - (m + 4.0) * H2[n, m] + \
                    (H3[n, m] * (n + m + 6.0) * (n - m - 4.0)) / 8.0
    return H1, H2, H3


ZH = _zernike_coeffs()


def zernike(p):
    H, W = p.shape
    rad = float(min(W, H))
    S = p.sum()
    ii = torch.arange(W, dtype=torch.float64).reshape(1, W) + 1
    jj = torch.arange(H, dtype=torch.float64).reshape(H, 1) + 1
    cx = (ii * p).sum() / S
    cy = (jj * p).sum() / S
    x = (ii - cx) / rad
    y = (jj - cy) / rad
    r2 = x * x + y * y
    r = torch.sqrt(r2)
    rd = r.detach()
    mask = ((rd >= EPS) & (rd <= 1.0)).to(torch.float64)
    rs = torch.where(mask > 0, r, torch.ones_like(r))
    r2s = rs * rs
    f = p / S * mask
    ct, st = x / rs, y / rs
    R = [torch.ones_like(rs)]
    for n in range(1, 16):
        R.append(rs * R[-1])
    cs, ss = [ct], [st]
    for m in range(1, 16):
        cs.append(ct * cs[-1] - st * ss[-1])
        ss.append(ct * ss[-1] + st * cs[-2])
    H1, H2, H3 = ZH
    out = []
    for n in range(16):
        Rv = {}
        Rnmp2 = Rnmp4 = None
        for m in range(n, -1, -2):
            if m == n:
                v = R[n]
                Rnmp4 = v
            elif m == n - 2:
                v = n * R[n] - (n - 1) * R[n - 2]
                Rnmp2 = v
            else:
                v = H1[n, m] * Rnmp4 + (H2[n, m] + H3[n, m] / r2s) * Rnmp2
                Rnmp4 = Rnmp2
                Rnmp2 = v
            Rv[m] = v
        for m in range(n % 2, n + 1, 2):
            ar = ((n + 1) / math.pi) * (f * Rv[m] * cs[m]).sum()
            ai = -((n + 1) / math.pi) * (f * Rv[m] * ss[m]).sum()
            out.append(torch.sqrt(ar * ar + ai * ai))
    return torch.stack(out)


def pixstats(p):
    v = p.reshape(-1)
    n = v.numel()
    s = torch.sort(v).values
    med = (s[n // 2 - 1] + s[n // 2]) / 2 if n % 2 == 0 else s[n // 2]
    return torch.stack([v.mean(), med, v.std(unbiased=True), s[0], s[-1]])


def fractal(p):
    H, W = p.shape
    K = min(W, H) // 5
    step = max(1, K // 20)
    out = [torch.zeros((), dtype=torch.float64) for _ in range(20)]
    b = 0
    for k in range(1, K, step):
        if b >= 20:
            break
        s = (p[:-k, :] - p[k:, :]).abs().sum() + (p[:, :-k] - p[:, k:]).abs().sum()
        out[b] = s / (W * (W - k) + H * (H - k))
        b += 1
    return torch.stack(out)


def gini(p):
    v = p.reshape(-1)
    v = v[v.detach() > 0]
    c = v.numel()
    if c <= 1:
        return torch.zeros(1, dtype=torch.float64)
    mean = v.sum() / c
    s = torch.sort(v).values
    i = torch.arange(1, c + 1, dtype=torch.float64)
    g = ((2.0 * i - c - 1.0) * s).sum()
    return (g / (mean * c * (c - 1))).reshape(1)


FAMILIES = {"Zernike Coefficients": zernike, "Pixel Intensity Statistics": pixstats,
            "Fractal Features": fractal, "Gini Coefficient": gini}


def features(img, groups):
    """The plan's features of one image, in plan order (groups: 'Alg (chain)')."""
    cache = {}

    def plane(chain):
        key = tuple(chain)
        if key not in cache:
            cache[key] = img if not chain else TRANSFORMS[chain[-1]](plane(chain[:-1]))
        return cache[key]

    out = []
    for g in groups:
        alg, ch = g.split(" (", 1)
        out.append(FAMILIES[alg](plane(chain_of("(" + ch))))
    return torch.cat(out)


def wnd(tfeat, Xtrain_n, y, C, w, mins, maxs):
    """classify2 marginal probabilities of one test feature vector."""
    rng = (maxs - mins)
    ok = rng >= EPS
    tv = torch.where(torch.isnan(tfeat), torch.zeros_like(tfeat), tfeat)
    # signatures::normalize's branches (0 below the range, 100 above it, the
    # quotient inside the closed range): at a value equal to max the derivative
    # is the quotient's (a clamp would split it between the two sides)
    t = 100 * ((tv - mins) / torch.where(ok, rng, 1.0))
    t = torch.where(tv > maxs, torch.full_like(t, 100.0), t)
    t = torch.where(ok & ~(tv < mins) & ~torch.isnan(tfeat), t, torch.zeros_like(t))
    keep = w.detach() >= EPS
    d = ((w[keep] ** 2) * (t[keep] - Xtrain_n[:, keep]) ** 2).sum(1)
    sims = []
    for c in range(1, C + 1):
        sel = (y == c) & (d.detach() >= EPS)
        sims.append((d[sel] ** -5).mean() if sel.any() else torch.zeros((), dtype=torch.float64))
    S = torch.stack(sims)
    return S / S.sum()


def normalize_train(X, mins, maxs):
    rng = maxs - mins
    Xn = 100 * ((X - mins) / np.where(rng >= EPS, rng, 1.0))
    Xn = np.where(np.isnan(X) | (X < mins) | (rng < EPS), 0.0, np.where(X > maxs, 100.0, Xn))
    return Xn
