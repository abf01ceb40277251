"""Multi-GPU use of the feature path: images are independent, so ranks are
replicas that each extract a contiguous shard of the image list; the rows are
gathered afterwards (no collective inside the data path).  The reference's own
equivalent is several wndchrm processes sharing one dataset through locked
.sig files (src/wndchrm_src/WORMfile.h) or a multiprocessing pool
(wndcharm/utils.py:406-440)."""
import numpy as np


def shard(n, rank, world):
    """Contiguous, balanced [lo, hi) of n items for `rank` of `world`."""
    base, extra = divmod(n, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def extract_sharded(images, extract_fn, group=None):
    """Every rank extracts its shard with extract_fn(list_of_images) -> (k, F)
    rows; returns the full (n, F) matrix on every rank, in input order."""
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    lo, hi = shard(len(images), rank, world)
    rows = np.asarray(extract_fn(images[lo:hi])) if hi > lo else None
    if world == 1:
        return rows
    parts = [None] * world
    dist.all_gather_object(parts, (lo, rows), group=group)
    F = next(p[1].shape[1] for p in parts if p[1] is not None)
    out = np.zeros((len(images), F))
    for lo_r, r in parts:
        if r is not None:
            out[lo_r: lo_r + len(r)] = r
    return out


def max_over_ranks(seconds, group=None):
    """The slowest rank's time: a step ends when every replica has finished."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return seconds
    t = torch.tensor([float(seconds)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def wnd_finish(sums, counts):
    """classify2's last steps from the per-class sums of d^-5 and their counts
    (TrainingSet.cpp:2429-2586, as k_wnd_finish does them on the GPU): each
    class's similarity is its mean d^-5 (classes without a row are 0), the
    predicted class the first strictly largest (1-based; -1 when no class has
    a row), the marginal probabilities the similarities over their sum.
    Returns (probs (T, C), pred (T,), normalisation factor (T,))."""
    sums = np.asarray(sums, dtype=np.float64)
    counts = np.asarray(counts, dtype=np.int64)
    T, C = sums.shape
    sim = np.where(counts > 0, sums / np.maximum(counts, 1), 0.0)
    pred = np.full(T, -1, dtype=np.int32)
    best = np.zeros(T)
    for c in range(C):  # first strictly larger wins, in class order
        up = (counts[:, c] > 0) & (sim[:, c] > best)
        best = np.where(up, sim[:, c], best)
        pred = np.where(up, c + 1, pred)
    tot = np.zeros(T)
    for c in range(C):
        tot = tot + sim[:, c]
    with np.errstate(invalid="ignore", divide="ignore"):
        probs = sim / tot[:, None]
    return probs, pred, tot


def wnd_classify_sharded(engine, train_shard, labels_shard, n_classes, weights, mins, maxs, test, group=None,
                         sums_fn=None):
    """classify2 with the training rows sharded across ranks: every rank takes
    its shard's per-class sums of d^-5 and counts for all test rows
    (Engine.wnd_class_sums, wc_wnd_class_sums), one all-reduce adds them, and
    every rank finishes the same probabilities and classes (wnd_finish).  The
    weights and ranges (wnd_fit on the whole set) are the same on every rank.
    sums_fn(train, labels, C, w, mn, mx, test) -> (sums, counts) replaces the
    engine call where a test runs the exchange without a GPU."""
    import torch
    import torch.distributed as dist
    fn = sums_fn if sums_fn is not None else engine.wnd_class_sums
    if len(train_shard):
        sums, counts = fn(train_shard, labels_shard, n_classes, weights, mins, maxs, test)
    else:
        sums = np.zeros((len(test), n_classes))
        counts = np.zeros((len(test), n_classes), dtype=np.int64)
    if dist.is_initialized() and dist.get_world_size(group) > 1:
        ts = torch.from_numpy(np.ascontiguousarray(sums))
        tc = torch.from_numpy(np.ascontiguousarray(counts))
        dist.all_reduce(ts, op=dist.ReduceOp.SUM, group=group)
        dist.all_reduce(tc, op=dist.ReduceOp.SUM, group=group)
        sums, counts = ts.numpy(), tc.numpy()
    probs, pred, _ = wnd_finish(sums, counts)
    return probs, pred


def class_means(sums, counts):
    """Per-label means of the exchanged sums (0 where a label has no row), as
    wc_wnd_fit divides them."""
    counts = np.asarray(counts, dtype=np.int64)
    with np.errstate(invalid="ignore", divide="ignore"):
        m = np.asarray(sums, dtype=np.float64) / counts[:, None].astype(np.float64)
    return np.where(counts[:, None] > 0, m, 0.0)


def wnd_fit_sharded(engine, train_shard, labels_shard, n_classes, frac=0.15, group=None, stats_fn=None,
                    fisher_fn=None):
    """wnd_fit (TrainingSet::normalize + SetFisherScores) with the training
    rows sharded across ranks: each rank's min / max and label counts, one
    MIN / MAX / SUM all-reduce; its per-label sums of the normalised values,
    one SUM all-reduce (the class means); its per-label sums of squared
    deviations, one SUM all-reduce; then the Fisher weights (wc_wnd_fisher) on
    every rank.  Returns (weights, mins, maxs), the same on every rank.
    stats_fn(stage, train, labels, C, mins, maxs, means) and
    fisher_fn(C, frac, sums, counts, sq) replace the engine calls where a test
    runs the exchange without a GPU."""
    import torch
    import torch.distributed as dist
    stats = stats_fn if stats_fn is not None else (
        lambda st, X, y, C, mn=None, mx=None, me=None: engine.wnd_fit_stats(st, X, y, C, mn, mx, me))
    fisher = fisher_fn if fisher_fn is not None else engine.wnd_fisher
    C = int(n_classes)
    multi = dist.is_initialized() and dist.get_world_size(group) > 1

    def reduce(a, op):
        if not multi:
            return a
        t = torch.from_numpy(np.ascontiguousarray(a))
        dist.all_reduce(t, op=op, group=group)
        return t.numpy()

    mins, maxs, counts = stats(0, train_shard, labels_shard, C)
    mins = reduce(mins, dist.ReduceOp.MIN if multi else None)
    maxs = reduce(maxs, dist.ReduceOp.MAX if multi else None)
    counts = reduce(counts, dist.ReduceOp.SUM if multi else None)
    sums = reduce(stats(1, train_shard, labels_shard, C, mins, maxs), dist.ReduceOp.SUM if multi else None)
    means = class_means(sums, counts)
    sq = reduce(stats(2, train_shard, labels_shard, C, mins, maxs, means), dist.ReduceOp.SUM if multi else None)
    return fisher(C, frac, sums, counts, sq), mins, maxs
