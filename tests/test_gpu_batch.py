"""Batched persistent launches: uneven stacks, sensitivity sweeps, CUDA graphs.

Every batched result must equal the single-stack path (which is itself pinned
to the reference) within float32 reordering differences of the temporal sums.
"""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from conftest import rel_err
from nanopyx_gb300 import engine
from nanopyx_gb300.synthetic import blinking_stack, emitters_for_density

pytestmark = pytest.mark.gpu


def _stacks():
    rng = np.random.default_rng(7)
    specs = []
    for k, (H, W, T, m, corr) in enumerate([(64, 64, 23, 2, "AVG"), (48, 80, 17, 5, "VAR"),
                                            (96, 40, 31, 4, "TAC2"), (33, 21, 9, 5, ("AVG", "VAR")),
                                            (128, 128, 12, 4, "AVG"), (20, 36, 40, 3, "TAC2")]):
        x = blinking_stack(T, H, W, emitters_for_density(H, W, 0.006), seed=100 + k)
        specs.append((x, dict(magnification=m, radius=float(rng.choice([1.0, 1.5, 2.0])),
                              sensitivity=1, temporal_correlation=corr,
                              frames_per_timepoint=int(rng.choice([0, 8])))))
    return specs


def test_uneven_batch_matches_single_calls():
    specs = _stacks()
    outs = engine.esrrf_batch([x for x, _ in specs], [kw for _, kw in specs])
    for (x, kw), o in zip(specs, outs):
        names = [kw["temporal_correlation"]] if isinstance(kw["temporal_correlation"], str) \
            else list(kw["temporal_correlation"])
        single = nx.esrrf_device(torch.from_numpy(x).cuda(), kw["magnification"], kw["radius"],
                                 kw["sensitivity"], kw["frames_per_timepoint"], names)
        assert o.shape == single.shape
        assert rel_err(o.cpu().numpy(), single.cpu().numpy()) <= 1e-5, kw


def test_sweep_matches_individual_reconstructions():
    x = blinking_stack(12, 48, 56, 16, seed=31)
    sens, radii = [1, 2, 3, 4, 1.5], [1.0, 1.5, 2.5]
    grid = nx.esrrf_parameter_sweep(x, magnification=4, sensitivities=sens, radii=radii)
    assert grid.shape == (5, 3, 192, 224)
    for i, s in enumerate(sens):
        for j, r in enumerate(radii):
            one = nx.eSRRF(x, 4, r, s, macro_pixel_correction=False)
            assert rel_err(grid[i, j], one) <= 1e-5, (s, r)


def test_graph_replay_equals_eager_and_is_repeatable():
    specs = _stacks()[:3]
    b = engine.EsrrfBatch()
    for x, kw in specs:
        b.add(x, **kw)
    eager = [o.clone() for o in b.run()]
    for o in b.outputs:
        o.zero_()
    g1 = [o.clone() for o in b.run(graph=True)]
    g2 = [o.clone() for o in b.run(graph=True)]
    for a, u, v in zip(eager, g1, g2):
        assert torch.equal(a, u) and torch.equal(u, v)


def test_frames_per_unit_does_not_change_the_result_beyond_rounding():
    x = blinking_stack(40, 64, 64, 24, seed=41)
    outs = []
    for fpu in (4, 40):
        b = engine.EsrrfBatch()
        b.add(x, 5, 1.5, 2, 0, ("VAR", "TAC2"), frames_per_unit=fpu)
        outs.append(b.run()[0].cpu().numpy())
    # different frame chunkings only change the float32 rounding of the
    # streamed moments (Welford updates within a chunk, pairwise merges across
    # chunks), which stays at the level of a few float32 ulps of the deviations
    assert rel_err(outs[0][0], outs[1][0]) <= 1e-5
    assert rel_err(outs[0][1], outs[1][1]) <= 1e-5


@pytest.mark.parametrize("m", [2, 4, 5])
def test_second_tiling_gives_identical_results(m):
    """The alternative tiling (one producer warp group fewer) only changes who
    prepares the gradient tiles: with the same frame chunking the results are
    bit-identical."""
    x = blinking_stack(12, 40, 72, 12, seed=70 + m)
    outs = []
    for v in (0, 1):
        b = engine.EsrrfBatch(tiles={(m, 3): v})
        b.add(x, m, 1.5, 2, 0, ("VAR", "TAC2"), frames_per_unit=6)
        b.add(x, m, 1.5, [1, 2], 0, "AVG", frames_per_unit=6)
        outs.append([o.clone() for o in b.run()])
        assert b.tiling[(m, 3)] == v
    for a, c in zip(*outs):
        assert torch.equal(a, c)


def test_tiling_autotuner_records_a_choice_per_kernel_key():
    x = blinking_stack(16, 64, 64, 20, seed=77)

    def build(tiles):
        b = engine.EsrrfBatch(tiles=tiles)
        b.add(x, 5, 1.5, 1, 0, "AVG")
        b.add(x, 2, 1.5, 1, 0, "TAC2")
        b.add(x, 3, 1.5, 1, 0, "VAR")
        return b

    rep = engine.tune_tiling(build, repeats=1, save=False)
    assert set(rep) == {"m2_J3", "m3_J3", "m5_J3"}
    assert rep["m3_J3"]["variant"] == 0 and 1 not in rep["m3_J3"]["ms"]  # one tiling only
    for k in ("m2_J3", "m5_J3"):
        assert rep[k]["variant"] in (0, 1) and set(rep[k]["ms"]) == {0, 1}
