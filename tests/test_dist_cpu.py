"""The multi-rank path on CPU: two gloo ranks shard a list of images, extract
their shards (with the CPU oracle standing in for the GPU worker) and gather
the rows; the result equals a single-process extraction, and the step time is
the slowest rank's."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

import synth_loader  # noqa: F401


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import oracle_features, oracle_lib
    from gpu_helpers import images
    from wndcharm.dist import extract_sharded, max_over_ranks
    imgs = images(seed=13, sizes=[(24, 20), (17, 23), (30, 18), (16, 16), (21, 25)])
    lib = oracle_lib()
    rows = extract_sharded(imgs, lambda part: np.stack([oracle_features(lib, a) for a in part]))
    t = max_over_ranks(1.0 + rank)
    q.put((rank, rows, t))
    dist.destroy_process_group()


def test_shard_bounds():
    from wndcharm.dist import shard
    for n in range(0, 13):
        for world in range(1, 5):
            spans = [shard(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(h - l for l, h in spans) - min(h - l for l, h in spans) <= 1


def test_two_gloo_ranks():
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from conftest import oracle_features, oracle_lib
    from gpu_helpers import images
    imgs = images(seed=13, sizes=[(24, 20), (17, 23), (30, 18), (16, 16), (21, 25)])
    lib = oracle_lib()
    ref = np.stack([oracle_features(lib, a) for a in imgs])
    for rank, rows, t in res:
        np.testing.assert_array_equal(rows, ref)
        assert t == 2.0


def _np_class_sums(X, y, C, w, mn, mx, T):
    """A numpy restatement of classify2's per-class sums (TrainingSet.cpp:2429-2586):
    the kept features normalised as signatures::normalize does, per-feature
    terms below DBL_EPSILON skipped, rows with d < DBL_EPSILON skipped."""
    eps = np.finfo(np.float64).eps
    keep = w >= eps
    rng = mx - mn

    def norm(A):
        with np.errstate(invalid="ignore", divide="ignore"):
            v = 100 * ((A - mn) / np.where(rng >= eps, rng, 1.0))
        v = np.where(A > mx, 100.0, v)
        return np.where(np.isnan(A) | (A < mn) | (rng < eps), 0.0, v)[:, keep]

    Xn, Tn, w2 = norm(X), norm(T), w[keep] ** 2
    sums = np.zeros((len(T), C))
    counts = np.zeros((len(T), C), dtype=np.int64)
    for t in range(len(T)):
        diff = np.abs(Tn[t] - Xn)
        diff = np.where(diff < eps, 0.0, diff)
        d = (w2 * diff * diff).sum(1)
        for c in range(1, C + 1):
            sel = (y == c) & (d >= eps)
            sums[t, c - 1] = (d[sel] ** -5.0).sum()
            counts[t, c - 1] = sel.sum()
    return sums, counts


def _wnd_worker(rank, world, port, data, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from wndcharm.dist import shard, wnd_classify_sharded
    xtr, ytr, xte, w, mn, mx = data
    lo, hi = shard(len(xtr), rank, world)
    probs, pred = wnd_classify_sharded(None, xtr[lo:hi], ytr[lo:hi], 5, w, mn, mx, xte,
                                       sums_fn=lambda *a: _np_class_sums(*a))
    q.put((rank, probs, pred))
    dist.destroy_process_group()


def test_wnd_training_rows_sharded_over_two_gloo_ranks():
    """WND-5 with the training rows split over two ranks and one all-reduce of
    the per-class sums and counts: every rank gets classify2's result for the
    whole training set (the oracle's), with a duplicated row that both
    the reference and the shards skip."""
    import socket
    from conftest import oracle_lib, oracle_wnd
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(301, 23, 120, 5, 6)
    xte[3] = xtr[10]  # distance 0 to one training row: skipped
    w, mn, mx, p_ref, pred_ref = oracle_wnd(oracle_lib(), xtr, ytr, xte, 5, 0.15)
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    data = (xtr, ytr, xte, w, mn, mx)
    procs = [ctx.Process(target=_wnd_worker, args=(r, 2, port, data, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, probs, pred in res:
        np.testing.assert_array_equal(pred, pred_ref)
        np.testing.assert_allclose(probs, p_ref, rtol=1e-12, atol=1e-15)


def test_wnd_finish_matches_the_rules():
    from wndcharm.dist import wnd_finish
    sums = np.array([[2.0, 6.0, 0.0], [1.0, 1.0, 0.0], [0.0, 0.0, 0.0]])
    counts = np.array([[1, 2, 0], [1, 1, 0], [0, 0, 0]])
    probs, pred, tot = wnd_finish(sums, counts)
    np.testing.assert_allclose(probs[0], [0.4, 0.6, 0.0])
    assert list(pred) == [2, 1, -1]  # ties: the first class; no rows: -1
    assert tot[0] == 5.0


FLT_MAX = float(np.finfo(np.float32).max)


def _np_fit_stats(stage, X, y, C, mins=None, maxs=None, means=None):
    """A numpy restatement of one process's fit statistics
    (TrainingSet::normalize + SetFisherScores, TrainingSet.cpp:2090-2324)."""
    F = X.shape[1]
    if stage == 0:
        ok = ~np.isnan(X) & (np.abs(X) <= FLT_MAX)
        mn = np.where(ok, X, np.inf).min(0)
        mx = np.where(ok, X, -np.inf).max(0)
        mn = np.where(np.isinf(mn), FLT_MAX, mn)
        mx = np.where(np.isinf(mx), -FLT_MAX, mx)
        counts = np.array([(y != 0).sum()] + [(y == c).sum() for c in range(1, C + 1)], dtype=np.int64)
        return mn, mx, counts
    rng = maxs - mins
    with np.errstate(invalid="ignore", divide="ignore"):
        v = 100 * ((X - mins) / np.where(rng >= np.finfo(np.float64).eps, rng, 1.0))
    v = np.where(X > maxs, 100.0, v)
    v = np.where(np.isnan(X) | (X < mins) | (rng < np.finfo(np.float64).eps), 0.0, v)
    out = np.zeros((C + 1, F))
    for c in range(0, C + 1):
        sel = (y != 0) if c == 0 else (y == c)
        if stage == 1:
            out[c] = v[sel].sum(0)
        elif c > 0:
            out[c] = ((v[sel] - means[c]) ** 2).sum(0)
    return out


def _np_fisher(C, frac, sums, counts, sq):
    from wndcharm.dist import class_means
    means = class_means(sums, counts)
    dev = ((means[1:] - means[0]) ** 2).sum(0)
    var = np.zeros(sums.shape[1])
    for c in range(1, C + 1):
        if counts[c] > 2:
            var = var + sq[c] / (counts[c] - 1)
    dev = dev / (C - 1) if C > 1 else dev * 0
    var = np.maximum(var / C, 0.000001)
    w = dev / var
    last = int(np.floor(frac * len(w) + 0.5))
    if last < len(w):
        thr = np.sort(w)[::-1][last]
        w = np.where(w < thr, 0.0, w)
    return w


def _fit_worker(rank, world, port, data, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from wndcharm.dist import shard, wnd_fit_sharded
    xtr, ytr = data
    lo, hi = shard(len(xtr), rank, world)
    w, mn, mx = wnd_fit_sharded(None, xtr[lo:hi], ytr[lo:hi], 5, 0.15, stats_fn=_np_fit_stats, fisher_fn=_np_fisher)
    q.put((rank, w, mn, mx))
    dist.destroy_process_group()


def test_wnd_fit_sharded_over_three_gloo_ranks():
    """The fit with the training rows split over three ranks (min / max, then
    sums, exchanged): the oracle's single-process weights, ranges and
    selection, with NaN and out-of-float-range values in the rows."""
    import socket
    from conftest import oracle_lib, oracle_wnd
    from wndcharm import synth
    xtr, ytr, xte, _ = synth.feature_vectors(400, 5, 150, 5, 8)
    xtr[3, 7] = np.nan
    xtr[10, 9] = 1e300
    w_ref, mn_ref, mx_ref, _, _ = oracle_wnd(oracle_lib(), xtr, ytr, xte, 5, 0.15)
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_fit_worker, args=(r, 3, port, (xtr, ytr), q)) for r in range(3)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, w, mn, mx in res:
        np.testing.assert_array_equal(mn, mn_ref)
        np.testing.assert_array_equal(mx, mx_ref)
        np.testing.assert_array_equal(w == 0, w_ref == 0)
        np.testing.assert_allclose(w, w_ref, rtol=1e-12, atol=0)
