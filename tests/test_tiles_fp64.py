"""The batched path on full-size tiles of the uneven-tile mixture, against
the FP64 oracle (the C restatement of the reference's generator.cpp:267-383
and simulator.cpp:235-363, pinned bit for bit to the reference's own build by
tests/test_oracle.py), run in the same test on the same tiles.

The tiles are taken from the benchmark's 256-tile mixture (seeds 1000 + i)
so that the inputs no small golden exercises are covered: fiber directions
uniform on the sphere, negative dn (a warning in the reference, allowed),
mu near 20 / mm, z sizes that are not multiples of 4, and 501-512 voxel
wide tiles.  Every tile runs 5 tilts x 9 polarizer angles (Slerp) in one
batch, with both march variants (per-thread and warp-cooperative); labels
and vectors must be bit-exact, images within 1e-4 relative per pixel and the
fused epa maps within 1e-3 of epa of the oracle's images."""

import os
import warnings

import numpy as np
import pytest

import parity
from fastpli_gb300 import synth
from fastpli_gb300.batch import TileBatch

# 34: dn = -0.0034, mu 18.4, 335 x 504 x 104
# 65: 478 x 512 x 67 (512 wide, Z % 4 = 3)
# 67: dn = -0.0040, 1908 fibers, 86 x 477 x 97
# 199: mu = 19.98, 327 x 501 x 58
# 234: 503 x 502 x 119, the largest of the picks
PICKS = (34, 65, 67, 199, 234)


def test_picked_tiles_cover_the_edge_inputs():
    params = {i: synth.tile_params(i) for i in PICKS}
    assert any(dn < -0.003 for _, _, dn, _ in params.values())
    assert any(mu > 19.9 for _, _, _, mu in params.values())
    assert sum(d[2] % 4 != 0 for d, _, _, _ in params.values()) >= 3
    assert any(max(d[:2]) == 512 for d, _, _, _ in params.values())


@pytest.fixture(scope="module")
def fp64(oracle_port):
    """Oracle labels, vectors, props and the 5 tilts' images of every pick."""
    threads = os.cpu_count() or 1
    out = {}
    for i in PICKS:
        t = synth.tile(i)
        lab, vec, props, _ = oracle_port.generate(t.dim, t.origin, t.voxel_size, t.bundles,
                                                  t.layers, n_threads=threads)
        imgs = [oracle_port.simulate(lab, vec, props, th, ph, n_threads=threads,
                                     **t.setup_kwargs())[0] for th, ph in t.tilts]
        out[i] = (t, lab, vec, props, imgs)
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("coop", [0, 1])
def test_tile_batch_matches_fp64(cuda, fp64, coop):
    torch = cuda
    tiles = [fp64[i][0] for i in PICKS]
    b = TileBatch(tiles, tiles[0].setup_kwargs(), epa=True).allocate()
    b.config = (0, 0, coop)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        b.run()
        torch.cuda.synchronize()
        b.warnings()
    worst = 0.0
    for t, i in enumerate(PICKS):
        _, lab, vec, props, imgs = fp64[i]
        glab = b.label(t).cpu().numpy()
        gvec = b.vector(t).cpu().numpy()
        n_lab = int(np.sum(glab != lab))
        n_vec = int(np.sum(gvec.view(np.uint32) != vec.view(np.uint32)))
        assert np.array_equal(b.props(t), props)
        for k, p in enumerate(b.pairs_of(t)):
            img = b.image(p).cpu().numpy()
            e = parity.image_errors(img, imgs[k])
            ep = parity.epa_errors([m.cpu().numpy() for m in b.epa_maps(p)],
                                   parity_epa(imgs[k]))
            parity.record(f"tiles/coop{coop}/tile{i}/tilt{k}", label_mismatch=n_lab,
                          vector_mismatch=n_vec, **e, **ep)
            worst = max(worst, e["max_rel"])
            assert e["max_rel"] <= parity.IMG_RTOL, (i, k, e)
            assert max(ep.values()) <= parity.EPA_TOL, (i, k, ep)
        assert n_lab == 0 and n_vec == 0, (i, n_lab, n_vec)
    print(f"tile batch (coop={coop}) vs FP64: max image rel err {worst:.3e}")
    b.close()


def parity_epa(img):
    import oracle
    return oracle.epa(img)
