"""Batched uneven stacks and the serving loop give the single-stack results bit for bit (needs a GPU)."""

import time

import numpy as np
import pytest

from conftest import gpu_ready

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_ready(), reason="needs a CUDA GPU")]


@pytest.fixture(scope="module")
def fddm(built_lib):
    import fastddm_gb300

    return fastddm_gb300


def _stacks():
    from fastddm_gb300.synthetic import Scene, make_stack

    specs = [(30, 64, 64, "uint16"), (17, 48, 40, "uint16"), (41, 96, 96, "uint8"), (9, 21, 17, "uint16"),
             (64, 128, 128, "uint16"), (25, 32, 96, "uint8")]
    return [make_stack(Scene(T, H, W, max(1, H * W // 82), 2.0, 150.0 if d == "uint8" else 2000.0, 0.4,
                             20.0 if d == "uint8" else 500.0, 0.0, d, 40 + i))
            for i, (T, H, W, d) in enumerate(specs)]


@pytest.mark.parametrize("mode", ["fft", "diff"])
def test_batch_equals_single_calls(fddm, mode):
    from fastddm_gb300.batch import ddm_batch

    stacks = _stacks()
    lags = [np.arange(1, s.shape[0]) for s in stacks]
    res = ddm_batch(stacks, lags, mode=mode)
    for s, lg, r in zip(stacks, lags, res):
        alone = fddm.ddm(s, lg, mode=mode)
        np.testing.assert_array_equal(r._data, alone._data)
        np.testing.assert_array_equal(r.kx, alone.kx)
        np.testing.assert_array_equal(r.ky, alone.ky)


def test_batch_graph_replay_equals_single_calls(fddm):
    """The batch captured into a CUDA graph: every replay rewrites each output with the single-call result,
    windowed and unwindowed stacks of several temporal kernel variants in one many-job launch per group."""
    import torch

    from fastddm_gb300.batch import BatchPlan, make_job

    dev = torch.device("cuda", 0)
    stacks = _stacks()
    lags = [np.arange(1, s.shape[0]) for s in stacks]
    windows = [fddm.window.blackman_harris(s.shape) if i % 2 else None for i, s in enumerate(stacks)]
    jobs = [make_job(s, lg, window=w, device=dev) for s, lg, w in zip(stacks, lags, windows)]
    plan = BatchPlan(jobs, "ff", dev, graph=True)
    alone = [fddm.ddm(s, lg, mode="fft", window=w)._data for s, lg, w in zip(stacks, lags, windows)]
    for _ in range(3):  # capture, then replays
        for j in jobs:
            j.out.fill_(float("nan"))
        outs = plan.run()
        torch.cuda.synchronize()
        for o, a in zip(outs, alone):
            np.testing.assert_array_equal(o.cpu().numpy(), a)
    assert plan._graph is not None


def test_batch_rejects_an_invalid_job_before_running(fddm):
    from fastddm_gb300 import _lib
    from fastddm_gb300.batch import BatchPlan, make_job
    import torch

    dev = torch.device("cuda", 0)
    good = make_job(_stacks()[0], range(1, 5), device=dev)
    bad = make_job(_stacks()[1], range(1, 5), device=dev)
    bad.nx = 17 * 3  # prime factor 17: unsupported
    with pytest.raises(_lib.FddmError, match="job 1"):
        BatchPlan([good, bad], "ff", dev)


def test_served_results_identical_alone_and_in_the_mix(fddm):
    import torch
    from fastddm_gb300.serving import DdmServer, GpuExecutor, Request, replay

    dev = torch.device("cuda", 0)
    stacks = _stacks()
    frames = [torch.from_numpy(s.astype(np.int32)).to(dev).to(torch.int16) for s in stacks]
    lags = [np.arange(1, s.shape[0]) for s in stacks]
    ex = GpuExecutor(0, "ff", n_streams=4, pool_bytes=2 << 30)
    server = DdmServer(ex, memory_budget=8 << 30, small_bytes=16 << 20)
    ex.clock_start()
    reqs = [Request(i, frames[i], lags[i], "fft", None, arrival=0.0) for i in range(len(stacks))]
    done = replay(server, reqs, time.perf_counter)
    assert sorted(r.rid for r in done) == list(range(len(stacks)))
    assert server.peak_inflight >= 2  # requests overlapped on the device
    assert server.batches >= 1  # small requests admitted together ran as one batch
    assert ex.pool.available == ex.pool.size  # every pooled workspace returned
    for i, s in enumerate(stacks):
        alone = fddm.ddm(s, lags[i], mode="fft")
        np.testing.assert_array_equal(server.fetch(i).cpu().numpy(), alone._data)
    assert all(r.latency > 0 for r in done)
