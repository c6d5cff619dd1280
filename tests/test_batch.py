"""Batched uneven tiles: host planning on CPU; on the GPU every tile's labels,
vectors and images must be bit-identical to the single-volume entry points,
and a CUDA-graph replay must reproduce the first run."""

import warnings

import numpy as np
import pytest

from fastpli_gb300 import batch as B
from fastpli_gb300 import synth
from fastpli_gb300.simulation import _Generator, _Simulator


def small_tiles(n=5, seed_base=500):
    out = []
    for i in range(n):
        t = synth.tile(i, seed_base=seed_base, n_fibers=12 + 5 * i)
        # shrink to test size, keep uneven shapes (odd z sizes included)
        rng = np.random.default_rng(seed_base + i)
        X, Y = (int(v) for v in rng.integers(17, 57, 2))
        Z = int(rng.integers(7, 31))
        t.dim = np.array([X, Y, Z])
        out.append(t)
    return out


def test_plan_is_host_only_and_consistent():
    tiles = small_tiles()
    b = B.TileBatch(tiles, dict(tiles[0].setup_kwargs()), epa=True)
    n = len(tiles)
    assert b.info.n_tiles == n and b.info.n_pairs == sum(len(t.tilts) for t in tiles)
    assert b.info.total_voxels == sum(int(np.prod(t.dim)) for t in tiles)
    offs = sorted(list(b.label_off) + list(b.vector_off) + list(b.image_off) + list(b.epa_off))
    assert all(o % 256 == 0 for o in offs)
    assert len(set(offs)) == len(offs)  # no two buffers share an offset
    assert b.info.arena_bytes > max(offs)
    sim = _Simulator()
    kw = tiles[0].setup_kwargs()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    steps = sum(sim.count_steps(t.dim, th, ph) for t in tiles for th, ph in t.tilts)
    assert b.steps == steps
    assert np.array_equal(b.props(2)[1:], B.TileBatch([tiles[2]], kw).props(0)[1:])
    b.close()


def test_symbols_exported():
    L = B.lib()
    for name in B.exported_symbols():
        assert hasattr(L, name)


@pytest.mark.gpu
@pytest.mark.parametrize("coop,wide", [(0, False), (1, False), (1, True)])
def test_batch_bit_identical_to_single_volume_path(cuda, coop, wide, monkeypatch):
    """Either march variant of the batch (per-thread or warp-cooperative),
    with 32-bit or (forced, FPGB_WIDE_INDEX=1) 64-bit index arithmetic, gives
    the single-volume path's bits."""
    torch = cuda
    if wide:
        monkeypatch.setenv("FPGB_WIDE_INDEX", "1")
    tiles = small_tiles()
    kw = tiles[0].setup_kwargs()
    b = B.TileBatch(tiles, kw, epa=True).allocate()
    b.config = (0, 0, coop)
    b.run()
    torch.cuda.synchronize()
    w = b.warnings()
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    for t, tile in enumerate(tiles):
        g = _Generator()
        g.set_volume(tile.dim, tile.origin, tile.voxel_size)
        g.set_fiber_bundles(tile.bundles, tile.layers)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            lab, vec, props = g.run_generation()
        assert np.array_equal(b.label(t).cpu().numpy(), lab), f"tile {t} labels"
        assert np.array_equal(b.vector(t).cpu().numpy().view(np.uint32), vec.view(np.uint32))
        for p in b.pairs_of(t):
            th, ph = b.tilts[p]
            ref = sim.run_simulation(tile.dim, lab, vec, props, th, ph)
            assert np.array_equal(b.image(p).cpu().numpy(), ref), f"tile {t} pair {p}"
    assert w["fp64_replays"] >= 0
    # every ray-block shape of the march gives the same bits
    before = [b.image(p).clone() for p in range(int(b.info.n_pairs))]
    for shape in range(1, len(B.TileBatch.SHAPES)):
        b.run(shape=shape)
        torch.cuda.synchronize()
        for p in range(int(b.info.n_pairs)):
            assert torch.equal(b.image(p), before[p]), (shape, p)
    b.set_shape(0)
    # a CUDA-graph replay reproduces the run exactly
    b.arena.zero_()
    b.replay()
    torch.cuda.synchronize()
    for p in range(int(b.info.n_pairs)):
        assert torch.equal(b.image(p), before[p])
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode,flip_z,step", [("NN", False, 1.0), ("Lerp", True, 1.0),
                                              ("Slerp", False, 0.7)])
def test_batch_modes_bit_identical_to_single_volume_path(cuda, mode, flip_z, step):
    """The other march instantiations of the batch: NN and Lerp, mirrored z,
    and a step size that makes the untilted rays no columns (the untilted
    launch then takes the general kernel) all give the single-volume path's
    bits."""
    torch = cuda
    tiles = small_tiles(n=4, seed_base=700)
    kw = dict(tiles[0].setup_kwargs(), interpolate=mode, flip_z=flip_z, step_size=step)
    b = B.TileBatch(tiles, kw, epa=True).allocate()
    b.run()
    torch.cuda.synchronize()
    sim = _Simulator()
    sim.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                      kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                      kw["flip_z"], kw["filter_rotations"])
    for t, tile in enumerate(tiles):
        lab, vec = b.label(t).cpu().numpy(), b.vector(t).cpu().numpy()
        for p in b.pairs_of(t):
            th, ph = b.tilts[p]
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                ref = sim.run_simulation(tile.dim, lab, vec, b.props(t), th, ph)
            assert np.array_equal(b.image(p).cpu().numpy(), ref), (mode, t, p)
    b.close()


@pytest.mark.gpu
def test_autotune_picks_a_config_and_results_do_not_change(cuda, tmp_path, monkeypatch):
    torch = cuda
    from fastpli_gb300 import autotune
    monkeypatch.setenv("FPGB_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    tiles = small_tiles(3, seed_base=700)
    b = B.TileBatch(tiles, tiles[0].setup_kwargs()).allocate()
    b.run(0, 1)
    torch.cuda.synchronize()
    ref = [b.image(p).clone() for p in range(int(b.info.n_pairs))]
    cfg, ms, table = autotune.tune(b, reps=1)
    assert cfg in table and ms > 0 and len(cfg) == 4
    assert {c[3] for c in table} == set(autotune.SHAPES)  # every ray-block shape was timed
    b.run()
    torch.cuda.synchronize()
    for p in range(int(b.info.n_pairs)):
        assert torch.equal(b.image(p), ref[p])
    cfg2, _, table2 = autotune.tune(b)
    assert cfg2 == cfg and table2 is None  # cached
    b.close()


@pytest.mark.gpu
def test_pipelined_host_call_matches_the_batch(cuda):
    """run_tiles_host (groups planned on a host thread while the previous
    group runs, images copied down on their own stream) returns, pair by
    pair, the images one TileBatch run gives."""
    torch = cuda
    tiles = small_tiles(7, seed_base=640)
    kw = tiles[0].setup_kwargs()
    b = B.TileBatch(tiles, kw).allocate()
    b.run()
    torch.cuda.synchronize()
    ref = [b.image(p).cpu().numpy() for p in range(int(b.info.n_pairs))]
    b.close()
    bufs = None
    for config in ((0, 2, 1, 3), (0, 1, 0, 0)):  # two calls, the second reusing the buffers
        imgs, st = B.run_tiles_host(tiles, kw, chunks=3, config=config, host_buffers=bufs)
        bufs = st["host_buffers"]
        assert st["groups"] == 3 and len(imgs) == len(ref)
        for a, r in zip(imgs, ref):
            assert np.array_equal(a, r)
