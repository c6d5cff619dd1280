"""fpgb_generate_tissue_noalloc: the voxelizer entry point for callers that
cannot allocate device memory (their GPU memory belongs to another
allocator, or they must not issue allocation calls).  Its scratch is a fixed
array inside the library; this file checks, through the C ABI, that it gives
exactly the results of fpgb_generate_tissue_device on two calls in a row
(the second reusing the scratch the first one left behind), that a call made
with the library's device pool released leaves the GPU's free memory
unchanged, and that a problem too large for the fixed scratch is refused
before any device work.

Named test_zz_* so that pytest collects it last."""

import warnings

import numpy as np
import pytest

import cases
from fastpli_gb300 import _native as N



def _inputs(c):
    flat = N.FlatFibers(c["bundles"], c["layers"])
    vol = N.make_volume(c["dim"], c["origin"], c["voxel_size"])
    return flat, vol


def _run(torch, fn, c, extra_ws=False):
    lib = N.load()
    flat, vol = _inputs(c)
    X, Y, Z = (int(v) for v in c["dim"])
    label = torch.full((X, Y, Z), -7, dtype=torch.int32, device="cuda")
    vector = torch.full((X, Y, Z, 3), 9.0, dtype=torch.float32, device="cuda")
    props = np.zeros((flat.n_props, 2))
    n_props = np.zeros(1, np.int64)
    w = N.Warnings()
    stream = torch.cuda.current_stream().cuda_stream
    if fn == "noalloc":
        rc = lib.fpgb_generate_tissue_noalloc(
            N.byref(vol), N.byref(flat.struct), 0, N.ptr(label), N.ptr(vector), N.ptr(props),
            flat.n_props, N.ptr(n_props), N.byref(w), stream)
    else:
        rc = lib.fpgb_generate_tissue_device(
            N.byref(vol), N.byref(flat.struct), 0, N.ptr(label), N.ptr(vector), N.ptr(props),
            flat.n_props, N.ptr(n_props), None, 0, N.byref(w), stream)
    N.check(rc)
    torch.cuda.synchronize()
    return label.cpu().numpy(), vector.cpu().numpy(), props, w.as_dict()


@pytest.mark.gpu
def test_noalloc_matches_device_entry_on_consecutive_calls(cuda):
    torch = cuda
    big = cases.synth_case(cases.crossing_small())   # two bundles, 307k voxels
    small = cases.gen_cases()["edges"]               # different shape and layers
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for c in (big, small, big):
            ref = _run(torch, "device", c)
            got = _run(torch, "noalloc", c)
            assert np.array_equal(got[0], ref[0])
            assert np.array_equal(got[1].view(np.uint32), ref[1].view(np.uint32))
            assert np.array_equal(got[2], ref[2])
            assert got[3] == ref[3]


@pytest.mark.gpu
def test_noalloc_call_allocates_no_device_memory(cuda):
    """With the library's cached pool released, any allocation on the call's
    path (the pool re-growing, a cudaMalloc) would lower the free device
    memory; a no-allocation call must leave it exactly where it was.  One
    call first loads the kernels' modules (lazy loading maps their code and
    the fixed scratch array the first time they are used)."""
    torch = cuda
    c = cases.synth_case(cases.crossing_small())
    lib = N.load()
    flat, vol = _inputs(c)
    X, Y, Z = (int(v) for v in c["dim"])
    label = torch.empty((X, Y, Z), dtype=torch.int32, device="cuda")
    vector = torch.empty((X, Y, Z, 3), dtype=torch.float32, device="cuda")
    props = np.zeros((flat.n_props, 2))
    w = N.Warnings()
    stream = torch.cuda.current_stream().cuda_stream

    def call():
        N.check(lib.fpgb_generate_tissue_noalloc(
            N.byref(vol), N.byref(flat.struct), 0, N.ptr(label), N.ptr(vector), N.ptr(props),
            flat.n_props, None, N.byref(w), stream))
        torch.cuda.synchronize()

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        call()
        first = label.clone()
        N.check(lib.fpgb_release_pool())
        torch.cuda.synchronize()
        free_before, _ = torch.cuda.mem_get_info()
        call()
        free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert torch.equal(label, first)


def test_scratch_limit_stated_in_the_header_matches_the_workspace_size():
    """The header and the design notes quote the fixed scratch as enough for
    about 220,000 short fiber segments; derive that from the workspace size
    the library computes, so the documented figure cannot drift."""
    lib = N.load()

    def ws(n_fibers):
        rng = np.random.default_rng(9)
        fibers = []
        for _ in range(n_fibers):
            start = rng.uniform(4, 28, 3)
            pts = start + np.cumsum(rng.normal(0, 0.3, (11, 3)), axis=0)  # 10 segments
            fibers.append(np.hstack([pts, np.full((11, 1), 0.5)]))
        c = dict(dim=np.array([32, 32, 32]), origin=np.zeros(3), voxel_size=1.0,
                 bundles=[fibers], layers=[[(1.0, 0.004, 1.0, "r")]])
        flat, vol = _inputs(c)
        return lib.fpgb_generate_workspace_size(N.byref(vol), N.byref(flat.struct))

    per_segment = (ws(2000) - ws(1000)) / 10000.0
    limit = (64 << 20) / per_segment
    assert 200_000 <= limit <= 240_000, (per_segment, limit)


def _oversize_case():
    """300,000 short segments in a 64^3 volume: the segment table alone is
    larger than the fixed scratch."""
    rng = np.random.default_rng(5)
    fibers = []
    for _ in range(3000):
        start = rng.uniform(4, 60, 3)
        pts = start + np.cumsum(rng.normal(0, 0.3, (101, 3)), axis=0)
        fibers.append(np.hstack([pts, np.full((101, 1), 0.5)]))
    return dict(dim=np.array([64, 64, 64]), origin=np.zeros(3), voxel_size=1.0,
                bundles=[fibers], layers=[[(1.0, 0.004, 1.0, "r")]])


def test_oversize_case_needs_more_than_the_scratch():
    c = _oversize_case()
    flat, vol = _inputs(c)
    assert N.load().fpgb_generate_workspace_size(N.byref(vol), N.byref(flat.struct)) > 64 << 20


@pytest.mark.gpu
def test_noalloc_rejects_problems_beyond_its_scratch(cuda):
    torch = cuda
    c = _oversize_case()
    flat, vol = _inputs(c)
    lib = N.load()
    # full-size output, so that nothing could land outside it in any case
    label = torch.empty((64, 64, 64), dtype=torch.int32, device="cuda")
    rc = lib.fpgb_generate_tissue_noalloc(
        N.byref(vol), N.byref(flat.struct), 1, N.ptr(label), None, None, 0, None, None,
        torch.cuda.current_stream().cuda_stream)
    assert rc == N.FPGB_EINVAL
    assert b"scratch" in lib.fpgb_last_error()
