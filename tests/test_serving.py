"""Serving loop: admission by HBM budget, continuous batching, failure
handling (host-side, with a fake runner on CPU), and on the GPU that a
request's result is the same alone and in a mix."""

import threading
import time
import types

import numpy as np
import pytest

from fastpli_gb300 import serving, synth


class FakeEvent:
    def __init__(self, t):
        self.t = t

    def query(self):
        return time.perf_counter() >= self.t

    def synchronize(self):
        while not self.query():
            time.sleep(0.001)


class FakeRunner:
    """Completes each batch after `delay` s; raises for requests whose tile is
    named 'boom' (launch) or 'late-boom' (collect)."""

    n_rho = 9

    def __init__(self, delay=0.01):
        self.delay = delay
        self.batches = []
        self.lock = threading.Lock()

    def launch(self, reqs, stream):
        if any(r.tile.name == "boom" for r in reqs):
            raise RuntimeError("injected launch failure")
        with self.lock:
            self.batches.append([r.rid for r in reqs])
        return [r.rid for r in reqs], FakeEvent(time.perf_counter() + self.delay)

    def collect(self, h, reqs, stream):
        if any(r.tile.name == "late-boom" for r in reqs):
            raise RuntimeError("injected collect failure")
        for r in reqs:
            r.result = {"rid": r.rid}


def tile(name="t", dim=(16, 16, 8)):
    return types.SimpleNamespace(name=name, dim=np.array(dim), origin=np.zeros(3),
                                 voxel_size=0.2, bundles=[[np.zeros((2, 4))]],
                                 layers=[[(1.0, 0.0, 0.0, "b")]])


def test_form_batch_respects_budget_and_order():
    reqs = [types.SimpleNamespace(nbytes=n) for n in (5, 3, 4, 1)]
    assert form(reqs, 8, 10) == [0, 1]      # 5+3 fits, +4 does not: stop (FIFO)
    assert form(reqs, 100, 3) == [0, 1, 2]  # max tiles
    assert form(reqs, 4, 10) == []          # head does not fit: wait


def form(reqs, free, mx):
    got = serving.form_batch(reqs, free, mx)
    return [reqs.index(r) for r in got]


def test_server_batches_and_completes_all():
    runner = FakeRunner(delay=0.02)
    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=1e12,
                                max_tiles=4, n_slots=2, runner=runner, streams=["s0", "s1"])
    with srv:
        reqs = [srv.submit(tile(), [(0, 0)]) for _ in range(20)]
        for r in reqs:
            assert r.wait(10)["rid"] == r.rid
    assert sum(len(b) for b in runner.batches) == 20
    assert max(len(b) for b in runner.batches) <= 4
    assert len(runner.batches) < 20  # requests arriving together were batched


def test_warm_up_runs_every_path_on_every_slot_before_serving():
    """start(warm=...) runs the warm tiles through the single-request runner
    one by one and through the batch runner together, on each stream slot,
    on the worker thread, and returns only when that is done; a warm-up
    failure is raised by start()."""
    class SlotRunner(FakeRunner):
        def launch(self, reqs, stream):
            with self.lock:
                self.batches.append((stream, len(reqs), threading.current_thread().name))
            return [r.rid for r in reqs], FakeEvent(time.perf_counter() + self.delay)

    batch, single = SlotRunner(0.005), SlotRunner(0.005)
    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=1e12,
                                max_tiles=8, n_slots=2, runner=batch, single_runner=single,
                                streams=["s0", "s1"])
    srv.start(warm=[tile(), tile(), tile()], warm_tilts=[(0, 0)])
    try:
        assert sorted(b[:2] for b in single.batches) == [("s0", 1)] * 3 + [("s1", 1)] * 3
        assert sorted(b[:2] for b in batch.batches) == [("s0", 3), ("s1", 3)]
        assert {b[2] for b in single.batches + batch.batches} == {"fpgb-server"}
        r = srv.submit(tile(), [(0, 0)])
        assert r.wait(10) is not None
    finally:
        srv.stop()

    class Broken(FakeRunner):
        def launch(self, reqs, stream):
            raise RuntimeError("injected warm-up failure")

    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=1e12,
                                runner=Broken(), streams=["s0"], n_slots=1)
    with pytest.raises(RuntimeError, match="warm-up failure"):
        srv.start(warm=[tile()])
    assert not srv._thread.is_alive()


def test_single_request_batches_use_the_single_runner():
    """A batch of one request goes to the single-request runner (the plain
    per-call path in production), larger batches to the batch runner."""
    batch, single = FakeRunner(delay=0.05), FakeRunner(delay=0.001)
    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=1e12,
                                max_tiles=8, n_slots=1, runner=batch, streams=["s"],
                                single_runner=single)
    with srv:
        first = srv.submit(tile(), [(0, 0)])
        first.wait(10)
        rest = [srv.submit(tile(), [(0, 0)]) for _ in range(6)]
        for r in rest:
            r.wait(10)
    assert single.batches[0] == [first.rid]
    assert all(len(b) == 1 for b in single.batches)
    assert all(len(b) > 1 for b in batch.batches) and batch.batches
    assert sum(len(b) for b in batch.batches + single.batches) == 7


def test_budget_limits_bytes_in_flight():
    runner = FakeRunner(delay=0.03)
    t = tile()
    nb = serving.estimate_bytes(t, np.zeros((1, 2)), 9)
    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=2.5 * nb,
                                max_tiles=16, n_slots=4, runner=runner, streams=list("abcd"))
    with srv:
        reqs = [srv.submit(t, [(0, 0)]) for _ in range(9)]
        for r in reqs:
            r.wait(10)
    assert max(len(b) for b in runner.batches) <= 2
    big = srv.submit(tile(dim=(4096, 4096, 64)), [(0, 0)])
    with pytest.raises(MemoryError):
        big.wait(1)


def test_failures_are_reported_per_request_and_server_survives():
    runner = FakeRunner(delay=0.005)
    srv = serving.ForwardServer({"filter_rotations": np.zeros(9)}, hbm_budget=1e12,
                                max_tiles=1, n_slots=1, runner=runner, streams=["s"])
    with srv:
        a = srv.submit(tile("boom"), [(0, 0)])
        b = srv.submit(tile("late-boom"), [(0, 0)])
        c = srv.submit(tile("ok"), [(0, 0)])
        with pytest.raises(RuntimeError, match="launch failure"):
            a.wait(5)
        with pytest.raises(RuntimeError, match="collect failure"):
            b.wait(5)
        assert c.wait(5)["rid"] == c.rid
    stats = serving.latency_stats([a, b, c])
    assert stats["n"] == 1


@pytest.mark.gpu
def test_result_same_alone_and_in_mix(cuda):
    tiles = [synth.tile(i, seed_base=900, n_fibers=20) for i in range(5)]
    for i, t in enumerate(tiles):
        t.dim = np.array([24 + 7 * i, 31, 11 + 3 * i])
    kw = tiles[0].setup_kwargs()
    with serving.ForwardServer(kw, hbm_budget=8e9, max_tiles=8, n_slots=2) as srv:
        alone = srv.submit(tiles[2], tiles[2].tilts)
        alone_out = alone.wait(60)
    assert alone.batch_size == 1  # the plain per-call kernels
    # the mix is queued before the server thread starts, so it is admitted as
    # one batch: the request compared below runs in the batched kernels
    srv = serving.ForwardServer(kw, hbm_budget=8e9, max_tiles=8, n_slots=2)
    mix = [srv.submit(t, t.tilts[: 1 + (i % 5)]) for i, t in enumerate(tiles)]
    mix.append(srv.submit(tiles[2], tiles[2].tilts))
    with srv:
        out = [r.wait(60) for r in mix]
    assert mix[-1].batch_size == len(mix)
    for (ta, da, ra), (tb, db, rb) in zip(alone_out["epa"], out[-1]["epa"]):
        assert np.array_equal(ta, tb) and np.array_equal(da, db) and np.array_equal(ra, rb)
