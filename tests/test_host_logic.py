"""Host-side logic that needs no GPU: input normalisation, argument checks,
Workflow wiring, the synthetic generator."""
import numpy as np
import pytest
import torch

import nanopyx_gb300 as nx
from nanopyx_gb300 import methods, synthetic
from nanopyx_gb300.liquid import LiquidEngine


def test_check_image_shapes_and_dtype():
    a = nx.check_image(np.ones((4, 5), dtype=np.uint16))
    assert a.shape == (1, 4, 5) and a.dtype == np.float32
    b = nx.check_image(np.zeros((2, 3, 4), dtype=np.float64))
    assert b.shape == (2, 3, 4) and b.dtype == np.float32
    with pytest.raises(ValueError):
        nx.check_image(np.zeros(5))
    with pytest.raises(ValueError):
        nx.check_image(np.zeros((1, 2, 3, 4)))
    t = nx.check_image(torch.zeros(3, 4, dtype=torch.float64))
    assert tuple(t.shape) == (1, 3, 4) and t.dtype == torch.float32


def test_value2array():
    assert np.array_equal(nx.value2array(1.5, 3), np.full(3, 1.5, np.float32))
    assert nx.value2array(np.array([1, 2]), 2).dtype == np.float32


def test_correlation_names_validated_before_any_device_work():
    with pytest.raises(ValueError, match="AVG, VAR or TAC2"):
        methods._corr_list("MAX")
    with pytest.raises(ValueError):
        methods._corr_list([])
    assert methods._corr_list(("VAR", "TAC2")) == ["VAR", "TAC2"]


def test_unimplemented_options_raise():
    # the Fourier interpolation runs the reference's default tiling and padding only
    with pytest.raises(NotImplementedError):
        nx.fht_space_interpolation(np.zeros((2, 4, 4), np.float32), 2, tile_size=128)
    with pytest.raises(NotImplementedError):
        nx.fht_space_interpolation(np.zeros((2, 4, 4), np.float32), 2, doMirrorPadding=False)


class _Add(LiquidEngine):
    def run(self, a, b, run_type=None):
        return self._run(a, b, run_type=run_type)

    def _run_cuda(self, a, b):
        return a + b


class _Split(LiquidEngine):
    def run(self, a, run_type=None):
        return self._run(a, run_type=run_type)

    def _run_cuda(self, a):
        return a, 2 * a


def test_workflow_prev_return_value_wiring():
    wf = nx.Workflow((_Split(), (np.array([1.0]),), {}),
                     (_Add(), ("PREV_RETURN_VALUE_0_0", "PREV_RETURN_VALUE_0_1"), {}))
    out = wf.calculate()
    assert np.array_equal(out[0], np.array([3.0]))
    with pytest.raises(TypeError):
        nx.Workflow((1, 2))


def test_synthetic_generator_deterministic_and_plausible():
    a = synthetic.blinking_stack(20, 32, 40, 10, seed=3)
    b = synthetic.blinking_stack(20, 32, 40, 10, seed=3)
    c = synthetic.blinking_stack(20, 32, 40, 10, seed=4)
    assert a.dtype == np.float32 and a.shape == (20, 32, 40) and a.flags.c_contiguous
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # background 100 photons/px: median close to 100
    assert 95 < float(np.median(a)) < 106
    assert synthetic.emitters_for_density(100, 100, 0.006) == 60


@pytest.mark.parametrize("T,fpt", [(500, 100), (450, 100), (23, 23), (30, 12), (7, 3), (1, 1),
                                   (10, 10), (100, 100), (99, 33)])
def test_upload_segments_tile_the_stack(T, fpt):
    segs = methods.upload_segments(T, fpt)
    n_tp = -(-T // fpt)
    assert len(segs) == n_tp
    flat = [s for tsegs in segs for s in tsegs]
    assert flat[0][0] == 0 and flat[-1][1] == T
    assert all(a < b for a, b in flat)
    assert all(flat[i][1] == flat[i + 1][0] for i in range(len(flat) - 1))
    for tp, tsegs in enumerate(segs):  # segments never straddle a timepoint
        assert tsegs[0][0] == tp * fpt and tsegs[-1][1] == min(T, (tp + 1) * fpt)


def test_parallel_host_copy_handles_strided_views():
    from nanopyx_gb300 import _hostio

    rng = np.random.default_rng(3)
    src = rng.random((7, 300, 200), dtype=np.float32)
    dst = np.empty_like(src)
    _hostio.par_copy(dst, src)
    assert np.array_equal(dst, src)
    res = np.zeros((2, 5, 400, 300), np.float32)
    out = rng.random((2, 400, 300), dtype=np.float32)
    _hostio.par_copy(res[:, 3], out)
    assert np.array_equal(res[:, 3], out) and not res[:, :3].any() and not res[:, 4:].any()
    with pytest.raises(ValueError):
        _hostio.par_copy(dst[:3], src)


def test_autotune_cache_roundtrip_and_unwritable_location(tmp_path, monkeypatch):
    from nanopyx_gb300 import engine

    path = tmp_path / "tune" / "autotune.json"
    monkeypatch.setattr(engine, "_CACHE_PATH", str(path))
    assert engine._store_fpu("GPU/152/x", 5, 3, 32)
    assert engine._store_fpu("GPU/152/x", 4, 2, 16)
    data = engine._load_cache()
    assert data["GPU/152/x"] == {"m5_J3": 32, "m4_J2": 16}
    blocker = tmp_path / "file"
    blocker.write_text("")
    monkeypatch.setattr(engine, "_CACHE_PATH", str(blocker / "sub" / "autotune.json"))
    with pytest.warns(UserWarning):
        assert not engine._store_fpu("GPU/152/x", 5, 3, 8)


def test_clock_sampler_reads_samples_through_a_pipe():
    import sys
    import time

    import bench

    fake = ("import time\n"
            "for k in range(100):\n"
            "    print('0, %d, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, %s' % "
            "(2070 if k % 3 else 1995, 'Active' if k == 1 else 'Not Active'), flush=True)\n"
            "    time.sleep(0.05)\n")
    cs = bench.ClockSampler(0, command=[sys.executable, "-c", fake])
    with cs:
        time.sleep(0.3)
    s = cs.summary()
    assert s is not None and s["samples"] >= 3
    assert s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]
    missing = bench.ClockSampler(0, command=["no-such-sampler-binary"])
    with missing:
        pass
    assert missing.summary() is None


def test_brent_search_agrees_with_scipy():
    """The lockstep Brent search finds the minimisers scipy.optimize.brent
    finds from the same two starting points (including a downhill walk into a
    flat region, as the error map's blur width takes for sigma <= 0)."""
    from scipy.optimize import brent

    from nanopyx_gb300.scoring import _lockstep_brent

    fns = [
        lambda x: (x - 1.3) ** 2 + 0.5,
        lambda x: np.cos(x) + 0.1 * x,
        lambda x: np.log1p((x - 4.2) ** 2),
        lambda x: max(x, 0.0) ** 2 + 1.0,       # flat for x <= 0
        lambda x: (x - 20.0) ** 2,              # minimum far beyond the bracket
    ]
    brack = (0.0, 3.4)
    got = _lockstep_brent([brack] * len(fns), lambda b: {i: fns[i](x) for i, x in b.items()})
    for f, g in zip(fns, got):
        ref = brent(f, brack=brack, maxiter=1000)
        assert abs(f(g) - f(ref)) <= 1e-12 * max(1.0, abs(f(ref)))
        if f(-1.0) != f(-2.0):  # a strict minimum: the same abscissa
            assert abs(g - ref) <= 1e-6 * max(1.0, abs(ref))
        else:
            assert g <= 0.0 and ref <= 0.0


@pytest.mark.parametrize("shape,kw", [((2, 2, 8, 8), dict(radius=1.5, PSF_ratio=2.8, voxel_ratio=4.0)),
                                      ((2, 6, 8, 8), dict(radius=2.5)),
                                      ((8, 8), {}), ((2, 3, 4, 8, 8), {})])
def test_esrrf3d_declines_like_the_reference(shape, kw, capsys):
    """_le_esrrf3d.pyx:36-48: a wrong rank or a radius too large for the
    volume prints the reference's warning and returns None (host side, before
    any device work); the reference itself is compared where it is built."""
    x = np.zeros(shape, np.float32)
    assert nx.eSRRF3D_ST(verbose=False).run(x, **kw) is None
    ours = capsys.readouterr().out
    assert ours.startswith("Warning")
    from oracle import ref_build

    if ref_build.available():
        ref = ref_build.load()["eSRRF3D_ST"](verbose=False).run(x, run_type="Threaded", **kw)
        assert ref is None and capsys.readouterr().out == ours
