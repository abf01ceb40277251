#!/usr/bin/env python
"""Benchmark: images/s of the 2919-feature (long) WND-CHARM plan on 512 x 512
uint16 (12-bit) images, the blob + grating workload with 4 classes (seed 1):
the batched mixed-precision form against the plain per-image FP64 form.

One step = one batch of B images through the whole plan.
  value : batched mixed-precision form, device-resident (inputs already in HBM,
          features left in HBM), CUDA events on the engine's stream around each
          step, L2 flushed between steps (outside the timed region);
  e2e   : the same form through the public API with host buffers (pinned input
          images in, host feature rows out), host<->device copies inside the
          timed region;
  forms : the FP64 form batched, and per image (one image per call, the
          plain per-image FP64 GPU form), on the same images.
The cpu_baseline leg runs the oracle on the first images of the batch and
reports the mixed form's per-family error against it.
--impl reference times the reference algorithm on the host CPU cores (the
oracle port, one image per thread) on the same workload.

Multi-GPU (torchrun): independent replicas, one per rank (the path shards by
image); the slowest rank's time defines the step.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "wnd-charm_gb300"))

import numpy as np  # noqa: E402

METRIC = "images/sec, 2919-feature set, 512^2 uint16: mixed vs FP64 GPU form at stated tol"
IMG = 512
WORKLOAD = "long plan (2919 features), %dx%d uint16 12-bit blob+grating, 4 classes, seed 1" % (IMG, IMG)
# the config object both arms print (the arm-specific set-up goes in top-level keys)
CONFIG = {"workload": WORKLOAD, "parallelism": "replicas",
          "l2": "GPU arm: flushed (256 MB write) between timed steps; CPU arm: not applicable"}


def clocks_sampler(stop, out):
    cmd = ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-i", os.environ.get("LOCAL_RANK", "0")]
    while not stop.is_set():
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=5)
            if r.returncode == 0 and r.stdout.strip():
                out.append([x.strip() for x in r.stdout.strip().split(",")])
        except Exception:
            pass
        stop.wait(0.2)


def summarize_clocks(samples):
    if not samples:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    sm = [float(s[0]) for s in samples if s[0].replace(".", "").isdigit()]
    mx = [float(s[1]) for s in samples if s[1].replace(".", "").isdigit()]
    reasons = set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for s in samples:
        for k, n in enumerate(names):
            if len(s) > 4 + k and s[4 + k].lower().startswith("active"):
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons)}


def make_images(n, seed=1):
    from wndcharm import synth
    per = (n + 3) // 4
    imgs, _ = synth.config2(n_per_class=per, size=IMG, seed=seed)
    order = [c * per + i for i in range(per) for c in range(4)][:n]  # interleave the classes
    return [imgs[k] for k in order]


def cpu_baseline(images, nthreads):
    sys.path.insert(0, os.path.join(REPO, "tests"))
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    ora = ctypes.CDLL(os.path.join(REPO, "oracle", "build", "libwc_oracle.so"))
    n = len(images)
    pix = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel() for a in images])
    offs = np.cumsum([0] + [a.size for a in images[:-1]]).astype(np.int64)
    ws = np.array([a.shape[1] for a in images], dtype=np.int32)
    hs = np.array([a.shape[0] for a in images], dtype=np.int32)
    out = np.zeros((n, 2919))
    D = ctypes.POINTER(ctypes.c_double)
    t0 = time.perf_counter()
    ora.wco_extract_std_batch(1, pix.ctypes.data_as(D), offs.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                              ws.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                              hs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n, 16, out.ctypes.data_as(D), nthreads)
    dt = time.perf_counter() - t0
    return n / dt, dt, out


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload == "short":
        return run_short(args, reference=True)
    if args.workload == "wnd":
        return run_wnd(args, reference=True)
    if args.workload == "grad":
        return run_grad(args, reference=True)
    nthreads = os.cpu_count() or 1
    # each timed step: one image per host thread on every host thread (the
    # reference's own model: one single-threaded process per image per core)
    per_step = nthreads
    warm = make_images(1, seed=99)
    for _ in range(args.warmup):
        cpu_baseline([w[:64, :64] for w in warm], 1)
    imgs = make_images(per_step)
    tot_imgs, tot_t = 0, 0.0
    for _ in range(args.steps):
        _, dt, _ = cpu_baseline(imgs, min(nthreads, per_step))
        tot_imgs += len(imgs)
        tot_t += dt
    v = tot_imgs / tot_t
    line = {"metric": METRIC, "value": v, "unit": "images/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * tot_t / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference", "config": dict(CONFIG), "images_per_step": per_step,
            "cpu_baseline": {"value": v, "unit": "images/s", "cores": nthreads, "kind": "port",
                             "sample": "%d images of %dx%d per step, one per host thread" % (per_step, IMG, IMG)},
            "e2e": {"value": v, "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def stage_work(name, B, precision="mixed", f14="exact"):
    """Algorithmic work per step of a stage on the long plan at 512^2, for the
    roofline of the dominant stage: (kind, amount) with kind 'bytes' (HBM),
    'fp64' (FP64 flops) or 'flops'; None where no model applies."""
    px = IMG * IMG
    planes_c = 12  # group C runs on 12 planes per image
    table = {
        # FP64 instructions: the coarseness search's local means and the
        # direction quotient and atan, about 45 FP64 operations per pixel
        "Tamura Textures": ("fp64", B * planes_c * px * 45),
        "Gabor Textures": ("bytes", B * px * 8 * 2),
        # three 2-D Chebyshev transforms per image (of the image and of its
        # Fourier plane, 512 x 512, and of its wavelet plane, 520 x 520), each
        # two n^3 products; a multiply and an add per term (FP64 and unfused in
        # both forms: the reference's rounding)
        "Chebyshev": ("fp64", B * 2 * 2 * (2 * IMG ** 3 + (2 * ((IMG + 9) // 2)) ** 3)),
        "Comb Moments": ("bytes", B * planes_c * px * 8),
        "Radon Coefficients": ("bytes", B * planes_c * px * 8),
        "Fractal Features": ("bytes", B * planes_c * px * 8),
        "PixStats+Gini (sort)": ("bytes", B * planes_c * px * 8 * 16),
    }
    if precision == "fp64" or f14 == "exact":
        # FP64 operations of Q, the Hessenberg reduction and the real-Schur QR for
        # f14, counted by an instrumented run of the oracle on this workload
        # (about 1.3 G per 512^2 image: 10/3 Ng^3 + 9 per touched element per
        # Francis step + 3 per nonzero Q term, summed over the 48 matrices); the
        # mixed form's pairs-of-floats chain computes them on the FP32 pipe
        table["Haralick Textures"] = ("fp64", B * 1.3e9)
    if precision == "fp64":
        # Zernike moments (the mixed form sums them in pairs of floats)
        table["Zernike Coefficients"] = ("fp64", B * 8 * px * 460)
    return table.get(name)


def fp64_peak_tflops(dev):
    """FP64 roof for the FP64-pipe stages, measured live: cuBLAS DGEMM 4096^3,
    best of 5 (CUDA events)."""
    import torch
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    best = None
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1000.0
        best = t if best is None else min(best, t)
    return 2 * 4096 ** 3 / best / 1e12


def run_tiles(args):
    """The batched uneven-size workload: images with independent sides from
    {64, 96, ..., 1024} (seed 2), each cut into 4 x 4 tiles as wndchrm samples
    them, all tiles of a step's images through the long plan in one call
    (wc_extract_samples: images go to the GPU once, tiles are cut there).
    Host images in, host rows out, CUDA events around each call."""
    import torch
    import wndcharm
    from wndcharm import synth
    B = min(args.batch, 32)
    n = B * (args.steps + args.warmup)
    sizes = synth.uneven_sizes(n, seed=2)
    rng = np.random.default_rng(2)
    imgs = [synth.blob_image(rng, i % 8, w, h, mean=320, sd=80, scale=16, maxval=4095).astype(np.uint16)
            for i, (w, h) in enumerate(sizes)]
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    eng = wndcharm.Engine(0, args.precision)
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    s = wndcharm.Sampling(tiles_x=4, tiles_y=4)
    t = 0.0
    l0 = 0
    for k in range(args.warmup + args.steps):
        batch = imgs[k * B:(k + 1) * B]
        if k == args.warmup:
            l0 = eng.launches
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        rows = eng.extract_samples(plan, batch, s)
        b.record(stream)
        b.synchronize()
        if k >= args.warmup:
            t += a.elapsed_time(b) / 1000.0
    tiles = 16 * B * args.steps
    px = sum(w * h for w, h in sizes[args.warmup * B:])
    # the same tiles one per call (the per-image loop wndchrm runs), on a sample
    loop_eng = wndcharm.Engine(0, args.precision)
    loop_eng.set_stream(stream.cuda_stream)
    sample = [t for im in imgs[args.warmup * B:args.warmup * B + 4] for t in wndcharm.tiles(im, 4, 4)]
    loop_eng.extract(plan, [sample[0]])
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for tl in sample:
        loop_eng.extract(plan, [np.ascontiguousarray(tl)])
    b.record(stream)
    b.synchronize()
    t_loop = a.elapsed_time(b) / 1000.0
    # the same loop with CUDA-graph replay (a tile shape is captured once the
    # tuner has settled and replayed for the image's remaining tiles)
    g_eng = wndcharm.Engine(0, args.precision)
    g_eng.set_stream(stream.cuda_stream)
    g_eng.set_option("graph", 1)
    g_eng.extract(plan, [sample[0]])
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for tl in sample:
        g_eng.extract(plan, [np.ascontiguousarray(tl)])
    b.record(stream)
    b.synchronize()
    t_graph = a.elapsed_time(b) / 1000.0
    print(json.dumps({"metric": "tiles/sec, 2919-feature set, 4x4 ROI tiles of uneven 64..1024 px uint16 images",
                      "value": tiles / t, "unit": "tiles/s", "images_per_s": B * args.steps / t,
                      "megapixels_per_s": px / t / 1e6, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1000 * t / args.steps, "higher_is_better": True, "dtype": "f32+f64",
                      "data": "synthetic", "gpu_launches": eng.launches - l0, "rows_per_step": int(rows.shape[0]),
                      "one_tile_per_call": {"value": len(sample) / t_loop, "unit": "tiles/s",
                                            "sample": "the 64 tiles of 4 images, one wc_extract_batch call each"},
                      "one_tile_per_call_graph": {"value": len(sample) / t_graph, "unit": "tiles/s",
                                                  "graphs": g_eng.graph_stats(),
                                                  "sample": "the same 64 calls with the engine option graph = 1"},
                      "batched_vs_one_tile_per_call": (tiles / t) / (len(sample) / t_loop),
                      "autotuned": {k: v[0] for k, v in eng.tuning().items()},
                      "config": {"workload": "uneven sides {64..1024} (seed 2), blob+grating, 8 classes, 4x4 tiles "
                                             "cut on the GPU", "images_per_step": B, "precision_form": args.precision,
                                 "io": "host images in, host rows out (inside the timed region)"}}))


WND_METRIC = "test vectors/sec, WND-5 (normalize + Fisher top 15% + classify2), 1e5 train x 1e4 test x 2919 features"
WND_CONFIG = {"workload": "WND-5 at scale: 100,000 train x 10,000 test fp64 vectors x 2919 features, 10 classes, "
                          "N(mu_cf, 1) with mu_cf ~ N(0, 0.5), seed 4",
              "parallelism": "replicas", "l2": "inputs (2.6 GB) larger than L2"}


def wnd_cpu(xtr, ytr, xte, C, nthreads, rows):
    """The oracle's WND-5 (the reference's arithmetic) on the host: one fit over
    all training rows, then `rows` test rows split over nthreads threads.
    Returns (fit s, classify s, probs, pred)."""
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    ora = ctypes.CDLL(os.path.join(REPO, "oracle", "build", "libwc_oracle.so"))
    N, F = xtr.shape
    D, I = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    w, mn, mx = np.zeros(F), np.zeros(F), np.zeros(F)
    p, pr, secs = np.zeros((rows, C)), np.zeros(rows, dtype=np.int32), np.zeros(2)
    te = np.ascontiguousarray(xte[:rows])
    ora.wco_wnd_mt(xtr.ctypes.data_as(D), N, F, ytr.ctypes.data_as(I), C, ctypes.c_double(0.15), te.ctypes.data_as(D),
                   rows, w.ctypes.data_as(D), mn.ctypes.data_as(D), mx.ctypes.data_as(D), p.ctypes.data_as(D),
                   pr.ctypes.data_as(I), nthreads, secs.ctypes.data_as(D))
    return secs[0], secs[1], p, pr


def run_wnd(args, reference=False):
    """The WND-5 workload at scale: one step = normalize + Fisher scores on the
    100,000 training vectors and classify2 of the 10,000 test vectors."""
    from wndcharm import synth
    C, T = 10, args.wnd_test
    xtr, ytr, xte, yte = synth.feature_vectors(args.wnd_train, T, 2919, C, 4)
    N, F = xtr.shape
    nth = os.cpu_count() or 1
    rows = nth * 16  # test rows of the CPU sample

    def cpu_sample():
        tf, tc, p, pr = wnd_cpu(xtr, ytr, xte, C, nth, rows)
        # the full job at the sample's rates: one fit, T rows over nth threads
        return T / (tf + tc * T / rows), tf, tc, p, pr

    if (args.wnd_train, args.wnd_test) != (100000, 10000):
        WND_CONFIG["workload"] += " (run at %d train x %d test)" % (args.wnd_train, args.wnd_test)

    if reference:
        vals, tot = [], 0.0
        for _ in range(args.steps):
            v, tf, tc, _, _ = cpu_sample()
            vals.append(v)
            tot += tf + tc * T / rows
        v = statistics.median(vals)
        print(json.dumps({"metric": WND_METRIC, "value": v, "unit": "test vectors/s", "n_gpus": 1, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "impl": "reference", "config": dict(WND_CONFIG),
                          "cpu_baseline": {"value": v, "unit": "test vectors/s", "cores": nth, "kind": "port",
                                           "sample": "one fit over the 100,000 training vectors plus %d test vectors "
                                                     "on %d threads per step, scaled to the 10,000" % (rows, nth)},
                          "e2e": {"value": v, "unit": "test vectors/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    import wndcharm
    stream = torch.cuda.Stream()
    engines = {k: wndcharm.Engine(0, k) for k in ("mixed", "fp64")}
    for e in engines.values():
        e.set_stream(stream.cuda_stream)
    X = torch.from_numpy(xtr).cuda()
    y = torch.from_numpy(ytr).cuda()
    Tt = torch.from_numpy(xte).cuda()
    dw, dmn, dmx = (torch.empty(F, dtype=torch.float64, device="cuda") for _ in range(3))
    dp = torch.empty((T, C), dtype=torch.float64, device="cuda")
    dpr = torch.empty(T, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def step(e):
        e.wnd_fit_device(X, y, C, 0.15, dw, dmn, dmx)
        e.wnd_classify_device(X, y, C, dw, dmn, dmx, Tt, dp, dpr)

    def timed(fn, k):
        tot, st = 0.0, []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            tot += a.elapsed_time(b) / 1000.0
            st.append(wndcharm.Engine.wnd_last_stats())
        return tot, st

    emx = engines["mixed"]
    for _ in range(max(3, args.warmup)):
        step(emx)
    stop, samples = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, samples), daemon=True)
    th.start()
    l0 = emx.launches
    t_dev, stats = timed(lambda: step(emx), args.steps)
    launches = emx.launches - l0
    p_mx, pr_mx = dp.cpu().numpy().copy(), dpr.cpu().numpy().copy()
    # end to end: pinned host arrays through the host-buffer entry points
    hx, hy, ht = (torch.from_numpy(a).pin_memory() for a in (xtr, ytr, xte))
    hxn, hyn, htn = hx.numpy(), hy.numpy(), ht.numpy()

    def step_e2e():
        # the reference's classification run: fit on the training rows, then
        # classify the test rows, each host array copied to the GPU once
        emx.wnd_fit_classify(hxn, hyn, C, htn, 0.15)

    step_e2e()
    t_e2e, _ = timed(step_e2e, args.steps)
    stop.set()
    th.join(timeout=10)
    clocks = summarize_clocks(samples)
    # the FP64 form on the same step
    t64, _ = timed(lambda: step(engines["fp64"]), max(1, min(args.steps, 2)))
    k64 = max(1, min(args.steps, 2))
    p64, pr64 = dp.cpu().numpy(), dpr.cpu().numpy()
    st = stats[-1]
    K = st[2]
    kern_s = st[4] / 1e9 if st[4] else None
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    peak = peaks.get("bf16_tflops", 1900.0)
    alg = 2.0 * T * N * K  # one multiply-add per (test, training, feature) term
    roof = {"kernel": "k_wnd_tc (tcgen05.mma, bf16 digits, FP32 accumulate)", "bound": "tensor",
            "achieved": alg / kern_s / 1e12 if kern_s else None, "peak": peak, "unit": "TFLOP/s",
            "frac": (alg / kern_s / 1e12) / peak if kern_s else None, "traffic": None,
            "peak_source": "measured" if peaks else "fallback",
            "algorithmic_flops_per_launch": alg, "kernel_ms": 1000 * kern_s if kern_s else None,
            "issued_tflops": st[5] / kern_s / 1e12 if kern_s else None,
            "issued_frac": st[5] / kern_s / 1e12 / peak if kern_s else None,
            "issued_note": "13 digit-pair bf16 products per term over padded sizes (exact digit arithmetic)"}
    v = T * args.steps / t_dev
    h2d = N * F * 8 + T * F * 8 + N * 4
    d2h = 3 * F * 8 + T * C * 8 + T * 4
    line = {"metric": WND_METRIC, "value": v, "unit": "test vectors/s",
            "mixed_vs_fp64": v / (T * k64 / t64), "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 digits (exact) + f32 pairs + f64", "data": "synthetic",
            "config": dict(WND_CONFIG), "precision_form": "mixed",
            "e2e": {"value": T * args.steps / t_e2e, "unit": "test vectors/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roof,
            "fp64_form": {"value": T * k64 / t64, "ms_per_step": 1000 * t64 / k64},
            "tensor_core": {"ran": bool(st[0]), "rows_rechecked_fp64": st[1], "weighted_features": K,
                            "ctas": st[3]},
            "vs_fp64_form": {"classes_identical": bool((pr_mx == pr64).all()),
                             "max_abs_prob_diff": float(np.abs(p_mx - p64).max())},
            "accuracy_vs_truth": float((pr_mx == yte).mean())}
    if not args.no_cpu_baseline:
        vc, tf, tc, pc, prc = cpu_sample()
        line["cpu_baseline"] = {"value": vc, "unit": "test vectors/s", "cores": nth, "kind": "port",
                                "sample": "one fit over the 100,000 training vectors (%.1f s) plus %d test vectors on "
                                          "%d threads (%.1f s), scaled to the 10,000" % (tf, rows, nth, tc)}
        line["vs_oracle"] = {"rows": rows, "classes_identical": bool((prc == pr_mx[:rows]).all()),
                             "max_abs_prob_diff": float(np.abs(pc - p_mx[:rows]).max())}
    print(json.dumps(line), flush=True)


SHORT_METRIC = "images/sec, 1059-feature set + WND-5 (30 train / 10 test), 256^2 uint8, 2 classes"
SHORT_CONFIG = {"workload": "short plan (1059 features), 2 classes x 20 uint8 256x256 blob+grating, seed 0; WND-5 "
                            "Fisher top 15%, trained on 30, tested on 10",
                "parallelism": "replicas", "l2": "GPU arm: inputs resident; CPU arm: not applicable"}


def short_data():
    from wndcharm import synth
    imgs, labels = synth.image_set(2, 20, 256, 256, seed=0, bits=8)
    tr = [i for i in range(40) if i % 20 < 15]
    te = [i for i in range(40) if i % 20 >= 15]
    order = tr + te  # training images first
    return [imgs[i] for i in order], labels[order].astype(np.int32)


def short_cpu(imgs, labels, nthreads):
    """The oracle on the host: the short plan on the 40 images (one per thread),
    then WND-5 fit on the first 30 rows and classify2 of the last 10."""
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    ora = ctypes.CDLL(os.path.join(REPO, "oracle", "build", "libwc_oracle.so"))
    n = len(imgs)
    pix = np.concatenate([np.ascontiguousarray(a, dtype=np.float64).ravel() for a in imgs])
    offs = np.cumsum([0] + [a.size for a in imgs[:-1]]).astype(np.int64)
    ws = np.array([a.shape[1] for a in imgs], dtype=np.int32)
    hs = np.array([a.shape[0] for a in imgs], dtype=np.int32)
    nf = ora.wco_plan_n_features(0)
    rows = np.zeros((n, nf))
    D, I = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    t0 = time.perf_counter()
    ora.wco_extract_std_batch(0, pix.ctypes.data_as(D), offs.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                              ws.ctypes.data_as(I), hs.ctypes.data_as(I), n, 8, rows.ctypes.data_as(D), nthreads)
    w, mn, mx = np.zeros(nf), np.zeros(nf), np.zeros(nf)
    p, pr = np.zeros((10, 2)), np.zeros(10, dtype=np.int32)
    tr = np.ascontiguousarray(rows[:30])
    te = np.ascontiguousarray(rows[30:])
    ytr = np.ascontiguousarray(labels[:30])
    ora.wco_wnd(tr.ctypes.data_as(D), 30, nf, ytr.ctypes.data_as(I), 2, ctypes.c_double(0.15), te.ctypes.data_as(D),
                10, w.ctypes.data_as(D), mn.ctypes.data_as(D), mx.ctypes.data_as(D), p.ctypes.data_as(D),
                pr.ctypes.data_as(I))
    return time.perf_counter() - t0, rows, p, pr


def run_short(args, reference=False):
    """The short plan with WND-5: one step = features of the 40 images (FP64
    form, as the plain reference method computes them), WND-5 fit on the 30
    training rows and classify2 of the 10 test rows."""
    imgs, labels = short_data()
    nth = os.cpu_count() or 1
    if reference:
        tot = 0.0
        for _ in range(args.steps):
            dt, _, _, _ = short_cpu(imgs, labels, nth)
            tot += dt
        v = 40 * args.steps / tot
        print(json.dumps({"metric": SHORT_METRIC, "value": v, "unit": "images/s", "n_gpus": 1, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                          "impl": "reference", "config": dict(SHORT_CONFIG),
                          "cpu_baseline": {"value": v, "unit": "images/s", "cores": nth, "kind": "port",
                                           "sample": "the whole step (40 images, one per thread; then WND-5)"},
                          "e2e": {"value": v, "unit": "images/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}), flush=True)
        return
    import torch
    import wndcharm
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSet()
    nf = plan.n_features
    eng = wndcharm.Engine(0, "fp64")
    stream = torch.cuda.Stream()
    eng.set_stream(stream.cuda_stream)
    host = torch.from_numpy(np.stack(imgs)).pin_memory()
    dev_imgs = host.cuda()
    W = wndcharm._lib
    L = wndcharm.lib()
    descs_dev = (W.wc_image_desc * 40)()
    descs_host = (W.wc_image_desc * 40)()
    for i in range(40):
        descs_dev[i] = W.wc_image_desc(dev_imgs[i].data_ptr(), W.WC_U8, 256, 256, 8, 1)
        descs_host[i] = W.wc_image_desc(host[i].data_ptr(), W.WC_U8, 256, 256, 8, 0)
    feat = torch.empty((40, nf), dtype=torch.float64, device="cuda")
    y = torch.from_numpy(labels[:30]).cuda()
    dw, dmn, dmx = (torch.empty(nf, dtype=torch.float64, device="cuda") for _ in range(3))
    dp = torch.empty((10, 2), dtype=torch.float64, device="cuda")
    dpr = torch.empty(10, dtype=torch.int32, device="cuda")
    out_host = torch.empty((40, nf), dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()

    def step_dev():
        wndcharm.check(L.wc_extract_batch(eng._h, plan.handle, descs_dev, 40, ctypes.c_void_p(feat.data_ptr()), 1))
        eng.wnd_fit_device(feat[:30], y, 2, 0.15, dw, dmn, dmx)
        eng.wnd_classify_device(feat[:30], y, 2, dw, dmn, dmx, feat[30:], dp, dpr)

    res = {}

    def step_e2e():
        wndcharm.check(L.wc_extract_batch(eng._h, plan.handle, descs_host, 40, ctypes.c_void_p(out_host.data_ptr()),
                                          0))
        rows = out_host.numpy()
        res["p"], res["pred"], _, _, _ = eng.wnd_fit_classify(rows[:30], labels[:30], 2, rows[30:], 0.15)

    def timed(fn, k):
        tot = 0.0
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            tot += a.elapsed_time(b) / 1000.0
        return tot

    for _ in range(max(3, args.warmup)):
        step_dev()
    stop, samples = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, samples), daemon=True)
    th.start()
    l0 = eng.launches
    t_dev = timed(step_dev, args.steps)
    launches = eng.launches - l0
    step_e2e()
    t_e2e = timed(step_e2e, args.steps)
    stop.set()
    th.join(timeout=10)
    line = {"metric": SHORT_METRIC, "value": 40 * args.steps / t_dev, "unit": "images/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t_dev / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(SHORT_CONFIG), "precision_form": "fp64",
            "e2e": {"value": 40 * args.steps / t_e2e, "unit": "images/s", "h2d_bytes_per_step": 40 * 256 * 256 + 30 * nf * 8 + 10 * nf * 8 + 30 * 4,
                    "d2h_bytes_per_step": 40 * nf * 8 + 3 * nf * 8 + 10 * 2 * 8 + 40},
            "gpu_launches": int(launches), "clocks": summarize_clocks(samples),
            "predicted": [int(v) for v in dpr.cpu().numpy()], "truth": [int(v) for v in labels[30:]]}
    if not args.no_cpu_baseline:
        dt, rows, p, pr = short_cpu(imgs, labels, nth)
        line["cpu_baseline"] = {"value": 40 / dt, "unit": "images/s", "cores": nth, "kind": "port",
                                "sample": "the whole step (40 images, one per host thread; then WND-5), %.1f s" % dt}
        sys.path.insert(0, os.path.join(REPO, "tests"))
        from parity import compare
        names = open(os.path.join(REPO, "tests", "golden", "names_short.txt")).read().splitlines()
        got = out_host.numpy()
        line["vs_oracle"] = {"feature_rows_within_rules": all(not compare(got[i], rows[i], names, rtol=1e-7,
                                                                          f14="exact") for i in range(40)),
                             "classes_identical": bool((res["pred"] == pr).all()),
                             "max_abs_prob_diff": float(np.abs(res["p"] - p).max())}
    print(json.dumps(line), flush=True)


GRAD_METRIC = ("test images/sec, WND-5 class-evidence maps (d p_c / d pixel, every class) and d p / d Fisher "
               "weights, 400 continuous features, 256^2 fp32")
GRAD_CONFIG = {"workload": "differentiation: 256 fp32 256x256 blob+grating images in [0, 1], 4 classes, seed 3; "
                           "WND-5 trained on 192, 400 Fisher-selected features of the continuous families "
                           "(Zernike, pixel statistics, fractal, Gini on nonnegative planes); 64 test images",
               "parallelism": "replicas", "l2": "host buffers through wc_wnd_grad (inputs staged each call)",
               "timing": "host clock around the public call (host images in, host maps out), bracketed by device "
                         "synchronisation: value and e2e are this one end-to-end measurement"}


def run_grad(args, reference=False):
    """One step = the class-evidence maps of the 64 test images: one forward
    pass (features + classify2), then for each of the 4 classes a backward
    pass to the pixels and the weights.  Beside it: central differences (h = 1e-3) on 64
    random pixels of 8 test images through the GPU forward."""
    from wndcharm import synth
    imgs, labels = synth.config4(n=256, size=256, seed=3)
    tr, te = list(range(192)), list(range(192, 256))
    nth = os.cpu_count() or 1
    if reference:
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no differentiation: its feature "
                          "extraction and classify2 have no backward pass to time"}), flush=True)
        return
    import torch
    import wndcharm
    from wndcharm.grad import WNDModel, continuous_groups
    plan = wndcharm.FeatureComputationPlan("continuous")
    for g in continuous_groups():
        plan.add(g)
    eng = wndcharm.Engine(0, "fp64")
    rows = eng.extract(plan, [imgs[i] for i in tr])
    ytr = labels[tr]
    w, mn, mx = eng.wnd_fit(rows, ytr, 4, 1.0)
    thr = np.sort(w)[::-1][399]
    w = np.where(w >= thr, w, 0.0)
    model = WNDModel(eng, plan, rows, ytr, 4, mn, mx)
    test = [imgs[i] for i in te]
    n = len(test)

    seeds = np.tile(np.eye(4)[None], (n, 1, 1))  # every class: the class-evidence maps

    def step():
        model.run(test, w, seed=seeds)

    for _ in range(max(3, args.warmup)):
        step()
    stop, samples = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, samples), daemon=True)
    th.start()
    l0 = eng.launches
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    launches = eng.launches - l0
    stop.set()
    th.join(timeout=10)
    # central differences on a sample: at h = 1e-3 (a step that crosses kinks
    # on most pixels of a 256^2 map: values ~1e-5 apart change rank, fractal
    # differences change sign) and at h = 1e-6 (few kinks; the forward pass's
    # rounding over 2h is the limit)
    probs, _, _ = model.run(test, w)
    pred = probs.argmax(1)
    nimg, npix = 8, 64
    seed = np.zeros((nimg, 4))
    seed[np.arange(nimg), pred[:nimg]] = 1.0
    _, gp, _ = model.run(test[:nimg], w, seed=seed)
    fdr = {}
    for h in (1e-3, 1e-6):
        rng = np.random.default_rng(7)
        fd, an = [], []
        for i in range(nimg):
            base = test[i].astype(np.float64)
            batch, pix = [], []
            for _ in range(npix):
                yy, xx = int(rng.integers(256)), int(rng.integers(256))
                pix.append((yy, xx))
                for sg in (1, -1):
                    a = base.copy()
                    a[yy, xx] += sg * h
                    batch.append(a)
            pb, _, _ = model.run(batch, w)
            for k, (yy, xx) in enumerate(pix):
                fd.append((pb[2 * k, pred[i]] - pb[2 * k + 1, pred[i]]) / (2 * h))
                an.append(gp[i][yy, xx])
        fd, an = np.array(fd), np.array(an)
        rel = np.abs(fd - an) / (np.abs(an) + 1e-6 * np.abs(an).max())
        fdr["h=%g" % h] = {"relative_error_quantiles_50_75_90_99": [float("%.3g" % x) for x in
                                                                    np.quantile(rel, [0.5, 0.75, 0.9, 0.99])],
                           "within_1e-3": int((rel < 1e-3).sum())}
    # the forward part alone on the host cores (the oracle: features of the
    # continuous groups + classify2): the reference has no backward pass
    cpu = None
    if not args.no_cpu_baseline:
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
        ora = ctypes.CDLL(os.path.join(REPO, "oracle", "build", "libwc_oracle.so"))
        D = ctypes.POINTER(ctypes.c_double)
        sample = test[:min(nth, n)]
        out = np.zeros(256)

        def one(a):
            pix = np.ascontiguousarray(a, dtype=np.float64)
            o = np.zeros(256)
            for g in continuous_groups():
                ora.wco_extract_group(g.encode(), pix.ctypes.data_as(D), 256, 256, 16, o.ctypes.data_as(D))

        import concurrent.futures
        t1 = time.perf_counter()
        with concurrent.futures.ThreadPoolExecutor(nth) as ex:
            list(ex.map(one, sample))
        dt = time.perf_counter() - t1
        cpu = {"value": len(sample) / dt, "unit": "test images/s (forward features only)", "cores": nth,
               "kind": "port", "sample": "the 882 continuous features of %d test images, one per host thread; the "
                                         "reference has no backward pass, so this times the forward alone" % len(sample)}
    v = n * args.steps / t
    line = {"metric": GRAD_METRIC, "value": v, "unit": "test images/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": dict(GRAD_CONFIG),
            "e2e": {"value": v, "unit": "test images/s", "h2d_bytes_per_step": 4 * (n * 256 * 256 * 8 + rows.nbytes),
                    "d2h_bytes_per_step": 4 * (n * 256 * 256 * 8 + n * 4 * 8 + w.nbytes)},
            "gpu_launches": int(launches), "clocks": summarize_clocks(samples),
            "features": {"plan": plan.n_features, "weighted": int((w > 0).sum())},
            "finite_differences": dict(fdr, pixels=nimg * npix, images=nimg,
                                       against="the predicted class's probability, float64 copies of the images"),
            "accuracy_on_test": float((pred + 1 == labels[te]).mean())}
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=128,
                    help="images per step (128: a quarter of the 4 x 128-image workload)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--f14", default="exact", choices=["exact", "pairs"],
                    help="mixed form's Haralick f14 chain: exact (FP64, bit-identical to the oracle) or pairs of floats")
    ap.add_argument("--per-image", type=int, default=8, help="images timed one per call in the FP64 form")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--wnd-train", type=int, default=100000, help="--workload wnd: training vectors")
    ap.add_argument("--wnd-test", type=int, default=10000, help="--workload wnd: test vectors")
    ap.add_argument("--no-forms", action="store_true", help="skip the FP64 comparison forms")
    ap.add_argument("--workload", default="512", choices=["512", "tiles", "wnd", "short", "grad"],
                    help="512: the 512x512 images (the headline line); tiles: uneven images "
                         "(sides 64..1024) cut into 4 x 4 tiles on the GPU; wnd: WND-5 at 1e5 x 1e4 x 2919; "
                         "short: the short plan with WND-5 on 40 256x256 uint8 images; one line each")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload == "tiles":
        return run_tiles(args)
    if args.workload == "wnd":
        return run_wnd(args)
    if args.workload == "short":
        return run_short(args)
    if args.workload == "grad":
        return run_grad(args)

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import wndcharm
    B = args.batch
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    nf = plan.n_features
    stream = torch.cuda.Stream()
    eng = wndcharm.Engine(local, args.precision)
    eng.set_option("f14_exact", 1 if args.f14 == "exact" else 0)
    eng.set_stream(stream.cuda_stream)
    imgs = make_images(B, seed=1 + rank)
    host = torch.from_numpy(np.stack(imgs).view(np.int16)).pin_memory()
    dev_imgs = host.to(dev)
    feat_dev = torch.empty((B, nf), dtype=torch.float64, device=dev)
    out_host = torch.empty((B, nf), dtype=torch.float64).pin_memory()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    W = wndcharm._lib
    descs_dev = (W.wc_image_desc * B)()
    descs_host = (W.wc_image_desc * B)()
    for i in range(B):
        descs_dev[i] = W.wc_image_desc(dev_imgs[i].data_ptr(), W.WC_U16, IMG, IMG, 16, 1)
        descs_host[i] = W.wc_image_desc(host[i].data_ptr(), W.WC_U16, IMG, IMG, 16, 0)
    L = wndcharm.lib()

    def step_dev(e=eng, n=B, descs=descs_dev):
        wndcharm.check(L.wc_extract_batch(e._h, plan.handle, descs, n, ctypes.c_void_p(feat_dev.data_ptr()), 1))

    def step_e2e():
        wndcharm.check(L.wc_extract_batch(eng._h, plan.handle, descs_host, B, ctypes.c_void_p(out_host.data_ptr()), 0))

    def timed(fn, k):
        tot = 0.0
        for _ in range(k):
            with torch.cuda.stream(stream):
                flush.zero_()
            stream.synchronize()
            if dist:
                dist.barrier()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            tot += a.elapsed_time(b) / 1000.0
        if dist:
            t = torch.tensor([tot], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            tot = float(t.item())
        return tot

    for _ in range(max(3, args.warmup)):
        step_dev()
    stream.synchronize()
    stop, samples = threading.Event(), []
    th = threading.Thread(target=clocks_sampler, args=(stop, samples), daemon=True)
    th.start()
    l0 = eng.launches
    t_dev = timed(step_dev, args.steps)
    launches = eng.launches - l0
    for _ in range(2):
        step_e2e()
    t_e2e = timed(step_e2e, args.steps)
    stop.set()
    th.join(timeout=10)
    clocks = summarize_clocks(samples)
    mixed_rows = out_host.numpy().copy()

    # the FP64 form on the same images: batched, and one image per call
    forms = None
    if not args.no_forms:
        e64 = wndcharm.Engine(local, "fp64")
        e64.set_stream(stream.cuda_stream)
        step64 = lambda: step_dev(e64, B, descs_dev)  # noqa: E731
        step64()
        ks = max(1, min(args.steps, 2))
        t64 = timed(step64, ks)
        npi = max(1, min(args.per_image, B))
        one = (W.wc_image_desc * 1)()
        one[0] = descs_dev[0]
        step_dev(e64, 1, one)
        tpi = 0.0
        for i in range(npi):
            one[0] = descs_dev[i]
            tpi += timed(lambda: step_dev(e64, 1, one), 1)
        v_mixed = world * B * args.steps / t_dev
        forms = {"mixed_batched": v_mixed, "fp64_batched": world * B * ks / t64,
                 "fp64_per_image": world * npi / tpi,
                 "mixed_vs_fp64_per_image": v_mixed / (world * npi / tpi),
                 "mixed_vs_fp64_batched": v_mixed / (world * B * ks / t64),
                 "fp64_per_image_sample": "%d images, one wc_extract_batch call each" % npi}
        del e64

    # per-stage profile (one extra step, outside the timed regions)
    eng.profile(True)
    step_dev()
    stream.synchronize()
    prof = eng.profile_report()
    timeline = eng.profile_timeline()
    eng.profile(False)
    # and one with the lanes serialised: every stage's own duration (what a
    # launch list shows, caches warm), for the roofline of the dominant stage
    eng.profile(True, serial=True)
    step_dev()
    stream.synchronize()
    prof_alone = {name: ms for name, ms, _ in eng.profile_report()}
    eng.profile(False)
    # the dominant stage: the largest share of the serialised step (each stage
    # timed alone, as in the ncu launch lists under profiles/); its roofline
    # uses that duration
    top = {n: ms for n, ms in prof_alone.items() if not n.startswith("host") and ":" not in n}
    tot_prof = sum(top.values()) or 1.0
    dname = max(top, key=top.get)
    dom = (dname, top[dname], 1)
    peaks = {}
    pk_path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    hbm = peaks.get("hbm_gbs", 6800.0)
    tfl = peaks.get("bf16_tflops", 1900.0)
    work = stage_work(dom[0], B, args.precision, args.f14)
    roof = {"stage": dom[0], "stage_ms_alone_per_step": dom[1], "stage_share": dom[1] / tot_prof,
            "bound": "hbm", "achieved": None, "peak": hbm, "unit": "GB/s", "frac": None, "traffic": None,
            "peak_source": "measured" if peaks else "fallback"}
    # DRAM bytes per image of the stage's kernels: constants taken from one ncu
    # capture each (dram__bytes_read.sum + dram__bytes_write.sum of the named
    # kernel on a smaller step of this workload), scaled by the images of this
    # step; not measured in this run
    traffic_per_image = {"Chebyshev": (287e6 / 16, "k_cheb_gemm at batch 16 (287 MB DRAM read+write)"),
                         "Haralick Textures": (6.26e9 / 32, "the real-Schur work queue k_har_qr_queue, the stage's "
                                                            "largest kernel, at batch 32 (6.26 GB DRAM read+write: "
                                                            "the matrices exceed the L2)")}
    if dom[0] in traffic_per_image:
        per, what = traffic_per_image[dom[0]]
        roof["traffic"] = per * B
        roof["traffic_source"] = "constant: one ncu capture of %s, scaled by images; bytes per step" % what
    if work:
        kind, amt = work
        sec = dom[1] / 1000.0
        if kind == "bytes":
            roof.update({"bound": "hbm", "achieved": amt / sec / 1e9, "peak": hbm, "unit": "GB/s"})
        elif kind == "fp64":
            p64 = fp64_peak_tflops(dev)
            roof.update({"bound": "fp64", "achieved": amt / sec / 1e12, "peak": p64, "unit": "TFLOP/s",
                         "peak_source": "measured live: cuBLAS DGEMM 4096^3"})
        else:
            roof.update({"bound": "tensor", "achieved": amt / sec / 1e12, "peak": tfl, "unit": "TFLOP/s"})
        roof["frac"] = roof["achieved"] / roof["peak"]
    roof["stage_choice"] = ("largest share of the step with the lanes serialised (engine profile, each stage "
                            "timed alone with CUDA events on the engine's stream); achieved uses that time")
    # the whole step against its floor: the FP64 families' algorithmic work at the
    # measured FP64 peak plus one read of every plane per scan family at HBM speed
    p64 = roof["peak"] if roof.get("bound") == "fp64" else fp64_peak_tflops(dev)
    fl = sum(w[1] for w in (stage_work(n, B, args.precision, args.f14) for n in ("Haralick Textures", "Chebyshev",
                                                                        "Zernike Coefficients")) if w)
    by = sum(stage_work(n, B)[1] for n in ("Tamura Textures", "Gabor Textures", "Comb Moments", "Radon Coefficients",
                                            "Fractal Features", "PixStats+Gini (sort)"))
    floor_ms = 1000.0 * (fl / (p64 * 1e12) + by / (hbm * 1e9))
    step_roof = {"fp64_flops_per_step": fl, "bytes_per_step": by, "fp64_peak_tflops": p64, "hbm_gbs": hbm,
                 "floor_ms_per_step": floor_ms, "frac": floor_ms / (1000 * t_dev / args.steps)}

    value = world * B * args.steps / t_dev
    e2e = world * B * args.steps / t_e2e
    line = {"metric": METRIC, "value": value, "unit": "images/s",
            "mixed_vs_fp64_per_image": forms["mixed_vs_fp64_per_image"] if forms else None,
            "mixed_vs_fp64_batched": forms["mixed_vs_fp64_batched"] if forms else None,
            "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * t_dev / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
            "data": "synthetic", "config": dict(CONFIG), "images_per_step": B, "precision_form": args.precision,
            "f14_chain": args.f14,
            "e2e": {"value": e2e, "unit": "images/s", "h2d_bytes_per_step": B * IMG * IMG * 2,
                    "d2h_bytes_per_step": B * nf * 8},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "roofline": roof, "step_roofline": step_roof,
            "forms": forms,
            "stages_ms": {n: round(ms, 3) for n, ms, _ in prof},
            "timeline_ms": {n: [round(a, 1), round(b, 1)] for n, a, b in timeline},
            "stages_alone_ms": {n: round(ms, 3) for n, ms in prof_alone.items()},
            "autotuned": {k: v[0] for k, v in eng.tuning().items()}}
    if rank == 0 and not args.no_cpu_baseline:
        nth = os.cpu_count() or 1
        ncpu = min(nth, B)
        v, dt, ref = cpu_baseline(imgs[:ncpu], nth)
        line["cpu_baseline"] = {"value": v, "unit": "images/s", "cores": nth, "kind": "port",
                                "sample": "%d images of %dx%d (the first of the batch), one per host thread, %.1f s"
                                % (ncpu, IMG, IMG, dt)}
        sys.path.insert(0, os.path.join(REPO, "tests"))
        from parity import compare_mixed, family_errors, compare
        names = open(os.path.join(REPO, "tests", "golden", "names_long.txt")).read().splitlines()
        errs, ok = {}, True
        for i in range(ncpu):
            fam = family_errors(mixed_rows[i], ref[i], names)
            for k, (r, g, w) in fam.items():
                r0, g0, w0 = errs.get(k, (0.0, 0.0, ""))
                errs[k] = (max(r0, r), max(g0, g), w if g >= g0 else w0)
            cmp = compare_mixed if args.precision == "mixed" else compare
            # f14: bit-identical to the oracle through the exact chain; range-checked
            # for the pairs-of-floats chain (its agreement is reported below)
            if cmp(mixed_rows[i], ref[i], names, f14="exact" if args.f14 == "exact" else "range"):
                ok = False
        from parity import f14_columns, f14_errors
        f14i = f14_columns(names)
        f14_agree, f14_abs, f14_rel = f14_errors(mixed_rows[:ncpu][:, f14i], ref[:ncpu][:, f14i])
        line["error_vs_oracle"] = {"images": ncpu, "tolerances_met": ok, "f14_agree_1e-6": f14_agree,
                                   "f14_max_abs": f14_abs, "f14_max_rel": f14_rel,
                                   "max_rel": {k: float("%.3g" % v[0]) for k, v in sorted(errs.items())},
                                   "max_rel_to_group_max": {k: float("%.3g" % v[1]) for k, v in sorted(errs.items())},
                                   "worst": {k: v[2] for k, v in sorted(errs.items()) if v[1] > 0}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
