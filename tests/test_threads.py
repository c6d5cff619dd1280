"""Host threads sharing the library: the device buffers the host-buffer
entry points cache between calls belong to the calling thread, so two Python
threads that call run_generation / run_simulation on the same (legacy
default) stream, with volumes that grow from call to call, never free or
overwrite each other's buffers.  Every result must be bit-identical to the
same call made alone."""

import threading
import warnings

import numpy as np
import pytest

from fastpli_gb300 import synth
from fastpli_gb300.simulation import _Generator, _Simulator

DIMS = [(24, 20, 12), (40, 36, 20), (64, 56, 28), (96, 88, 40)]


def _workloads():
    return [synth.crossing(seed=60 + i, n_per_bundle=10 + 8 * i, dim=d, n_points=6)
            for i, d in enumerate(DIMS)]


def _forward(w):
    g = _Generator()
    g.set_volume(w.dim, w.origin, w.voxel_size)
    g.set_fiber_bundles(w.bundles, w.layers)
    lab, vec, props = g.run_generation()
    kw = w.setup_kwargs()
    s = _Simulator()
    s.set_pli_setup(kw["step_size"], kw["light_intensity"], kw["voxel_size"], kw["wavelength"],
                    kw["tissue_refrection"], kw["interpolate"], kw["untilt_sensor_view"],
                    kw["flip_z"], kw["filter_rotations"])
    th, ph = synth.TILTS_5[1]
    img = s.run_simulation(w.dim, lab, vec, props, th, ph)
    return lab.copy(), vec.copy(), img.copy()


@pytest.mark.gpu
def test_two_threads_growing_volumes_on_the_default_stream(cuda):
    torch = cuda
    ws = _workloads()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        alone = [_forward(w) for w in ws]
    torch.cuda.synchronize()
    errors = []
    start = threading.Barrier(2)

    def worker(order):
        try:
            start.wait()
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                for _ in range(3):
                    for i in order:  # sizes grow, so each thread's buffers are re-grown
                        lab, vec, img = _forward(ws[i])
                        ref = alone[i]
                        if not (np.array_equal(lab, ref[0])
                                and np.array_equal(vec.view(np.uint32), ref[1].view(np.uint32))
                                and np.array_equal(img, ref[2])):
                            errors.append(f"volume {i} differs")
        except Exception as e:  # reported by the main thread
            errors.append(repr(e))

    threads = [threading.Thread(target=worker, args=(o,))
               for o in ([0, 1, 2, 3], [1, 2, 3, 0])]
    for t in threads:
        t.start()
    for t in threads:
        t.join(600)
    assert not any(t.is_alive() for t in threads)
    assert not errors, errors[:5]
