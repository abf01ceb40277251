"""CUDA-graph replay of repeated batch shapes (engine option "graph"): a
shape is captured the second time it is seen, once the launch-shape tuner
has settled, and replayed after that.  Every call's features must equal an
ungraphed engine's bit for bit, on new pixels each call, for one-image calls
(the per-tile loop), for a batch of uneven sizes, on the engine's default
(legacy) stream and on a caller's stream; a new shape is captured on its own;
setting an option drops the graphs."""
import numpy as np
import pytest

from gpu_helpers import images
import synth_loader  # noqa: F401

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,autotune", [("mixed", 1), ("fp64", 0)])
def test_one_image_calls_replay_identically(prec, autotune):
    import wndcharm
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSetLong()
    g, ref = wndcharm.Engine(0, prec), wndcharm.Engine(0, prec)
    for e in (g, ref):
        e.set_option("autotune", autotune)
    g.set_option("graph", 1)
    for k in range(8):
        img = images(seed=100 + k, sizes=[(72, 60)])
        np.testing.assert_array_equal(g.extract(plan, img), ref.extract(plan, img))
    st = g.graph_stats()
    assert st["captures"] == 1 and st["replays"] >= 4 and st["failures"] == 0, st
    # a second shape gets its own graph (once the tuner has settled its
    # launch shapes); the first keeps replaying, after one more capture if
    # the larger shape moved a device buffer its graph addresses
    for k in range(12):
        img = images(seed=200 + k, sizes=[(50, 90)] if k % 2 else [(72, 60)])
        np.testing.assert_array_equal(g.extract(plan, img), ref.extract(plan, img))
    st2 = g.graph_stats()
    assert 2 <= st2["captures"] <= 3 and st2["kept"] == 2 and st2["replays"] > st["replays"] + 3, st2
    g.set_option("graph", 1)
    assert g.graph_stats()["kept"] == 0


def test_uneven_batch_on_a_caller_stream():
    import torch
    import wndcharm
    plan = wndcharm.StdFeatureComputationPlans.getFeatureSet()
    s = torch.cuda.Stream()
    g, ref = wndcharm.Engine(0, "mixed"), wndcharm.Engine(0, "mixed")
    g.set_stream(s.cuda_stream)
    g.set_option("graph", 1)
    sizes = [(64, 64), (130, 70), (33, 97), (80, 80)]
    for k in range(7):
        imgs = images(seed=300 + k, sizes=sizes)
        np.testing.assert_array_equal(g.extract(plan, imgs), ref.extract(plan, imgs))
    st = g.graph_stats()
    assert st["captures"] == 1 and st["replays"] >= 2, st
