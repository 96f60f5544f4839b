"""Continuous-batching server: results alone == results in the mix."""
import threading
import time

import numpy as np
import pytest

from nanopyx_gb300.serve import ESRRFServer, serve_plain
from nanopyx_gb300.synthetic import blinking_stack

pytestmark = pytest.mark.gpu


def _requests():
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(7):
        H = int(rng.choice([32, 48, 64, 96]))
        W = int(rng.choice([40, 64, 80]))
        nb = int(rng.integers(1, 4))
        T_block = int(rng.choice([7, 12]))
        x = blinking_stack(nb * T_block, H, W, max(2, H * W // 200), seed=200 + k)
        blocks = [x[i * T_block:(i + 1) * T_block] for i in range(nb)]
        kw = dict(magnification=int(rng.choice([2, 4, 5])), radius=1.5, sensitivity=1,
                  temporal_correlation=["AVG", "VAR", "TAC2", ("VAR", "TAC2")][k % 4])
        reqs.append((blocks, kw))
    return reqs


def _same(a, b):
    if isinstance(a, tuple):
        return all(np.array_equal(u, v) for u, v in zip(a, b))
    return np.array_equal(a, b)


def test_results_alone_equal_results_in_the_mix():
    reqs = _requests()
    alone = serve_plain([b for b, _ in reqs], [kw for _, kw in reqs])
    with ESRRFServer(n_streams=4) as srv:
        handles = [srv.submit(b[0].shape[1], b[0].shape[2], len(b), **kw) for b, kw in reqs]

        def feeder():
            # interleave the blocks of all requests as they "arrive"
            for i in range(3):
                for h, (blocks, _) in zip(handles, reqs):
                    if i < len(blocks):
                        srv.push(h, blocks[i])
                time.sleep(0.002)

        t = threading.Thread(target=feeder)
        t.start()
        t.join()
        mixed = [h.result(timeout=120) for h in handles]
    for a, m_, h in zip(alone, mixed, handles):
        assert _same(a, m_)
        assert h.latency is not None and h.latency >= 0
    assert srv.admitted_max >= 2  # requests really overlapped


def test_tiny_budget_still_completes_in_order():
    reqs = _requests()[:3]
    alone = serve_plain([b for b, _ in reqs], [kw for _, kw in reqs])
    with ESRRFServer(hbm_budget=1, n_streams=2) as srv:
        hs = []
        for blocks, kw in reqs:
            h = srv.submit(blocks[0].shape[1], blocks[0].shape[2], len(blocks), **kw)
            for b in blocks:
                srv.push(h, b)
            hs.append(h)
        out = [h.result(timeout=120) for h in hs]
    assert srv.admitted_max == 1  # the budget admits one request at a time
    for a, b in zip(alone, out):
        assert _same(a, b)


def test_bad_requests_are_rejected_on_the_host():
    with ESRRFServer(n_streams=1) as srv:
        h = srv.submit(16, 16, 1, magnification=2)
        with pytest.raises(ValueError):
            srv.push(h, np.zeros((3, 16, 17), np.float32))
        srv.push(h, np.ones((3, 16, 16), np.float32))
        with pytest.raises(ValueError):
            srv.push(h, np.ones((3, 16, 16), np.float32))
        h.result(timeout=60)
        with pytest.raises(ValueError):
            srv.submit(16, 16, 1, temporal_correlation="MAX")
    with pytest.raises(RuntimeError):
        srv.submit(16, 16, 1)
