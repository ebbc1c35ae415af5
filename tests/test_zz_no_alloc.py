"""ncg_sd_eval_m2lnp_device_noalloc: the FP64 eval for callers that must not
allocate device memory while they evaluate.

Who needs it: a caller that keeps other CUDA streams busy while it evaluates
(cudaMalloc may synchronise the whole device and stall them), or a caller that
owns all device memory under a fixed budget and forbids allocations hidden in
library calls.  The entry point keeps its per-call scratch in a static 4 MiB
device array instead of allocating it.

The test calls it through the C-ABI twice in a row on different points and
compares each result with the regular device entry point
(ncg_sd_eval_m2lnp_device) on the same points, within the FP64 tolerance of the
other GPU tests (1e-10 relative); it checks that the device's free memory does
not change across the two calls and that oversize requests are refused.
This file sorts last so that a run stopping at its first failure has already
run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden, rel_err

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10


def test_noalloc_eval_matches_regular_entry_point(gpu):
    import torch

    ng = gpu
    from numcosmo_gb300 import _lib

    L = _lib.load()
    g = golden("vkde_st3_d16_n1024")
    sd = ng.StatsDistVKDE(ng.StatsDistKernelST(16, 3.0), ng.StatsDistCV.NONE)
    sd.set_sample(g["centres"])
    sd.prepare()

    pts_a = torch.tensor(g["points"], dtype=torch.float64, device="cuda")
    pts_b = torch.tensor(g["centres"][:700] + 0.25, dtype=torch.float64, device="cuda")
    ref_a = torch.empty(pts_a.shape[0], dtype=torch.float64, device="cuda")
    ref_b = torch.empty(pts_b.shape[0], dtype=torch.float64, device="cuda")
    out_a = torch.empty_like(ref_a)
    out_b = torch.empty_like(ref_b)
    torch.cuda.synchronize()

    # the regular entry point (allocates its scratch on demand)
    for x, r in ((pts_a, ref_a), (pts_b, ref_b)):
        _lib.check(L.ncg_sd_eval_m2lnp_device(sd._h, C.c_void_p(x.data_ptr()), x.shape[0], C.c_void_p(r.data_ptr())),
                   "ncg_sd_eval_m2lnp_device")
    sd.synchronize()

    free_before = torch.cuda.mem_get_info()[0]
    # two calls in a row of the no-allocation variant, on different inputs
    for x, o in ((pts_a, out_a), (pts_b, out_b)):
        _lib.check(L.ncg_sd_eval_m2lnp_device_noalloc(sd._h, C.c_void_p(x.data_ptr()), x.shape[0],
                                                      C.c_void_p(o.data_ptr())),
                   "ncg_sd_eval_m2lnp_device_noalloc")
    sd.synchronize()
    free_after = torch.cuda.mem_get_info()[0]

    assert rel_err(out_a.cpu().numpy(), ref_a.cpu().numpy()) < FP64_TOL
    assert rel_err(out_b.cpu().numpy(), ref_b.cpu().numpy()) < FP64_TOL
    assert rel_err(out_a.cpu().numpy(), g["m2lnp"]) < FP64_TOL
    assert free_after == free_before

    # the same call again: the shared array keeps the previous contents, results must not depend on them
    _lib.check(L.ncg_sd_eval_m2lnp_device_noalloc(sd._h, C.c_void_p(pts_a.data_ptr()), pts_a.shape[0],
                                                  C.c_void_p(out_b.data_ptr())), "noalloc")
    sd.synchronize()
    assert np.array_equal(out_b[: pts_a.shape[0]].cpu().numpy(), out_a.cpu().numpy())

    # requests beyond the static scratch are refused before any launch
    too_many = 262144 + 1
    with pytest.raises(ng.NcgError) as e:
        _lib.check(L.ncg_sd_eval_m2lnp_device_noalloc(sd._h, C.c_void_p(pts_a.data_ptr()), too_many,
                                                      C.c_void_p(out_a.data_ptr())), "noalloc")
    assert e.value.name == "NCG_ERR_INVALID_ARG"
    assert "static scratch" in str(e.value)


def test_noalloc_eval_capped_slicing(gpu):
    """Point counts whose regular kernel slicing would not fit the static array:
    the slice count is capped (90000 points: 3 slices -> 2) and at the largest
    accepted count (262144 points: one slice); both against the regular entry
    point within the FP64 tolerance."""
    import torch

    ng = gpu
    from numcosmo_gb300 import _lib

    L = _lib.load()
    g = golden("vkde_st3_d16_n1024")
    sd = ng.StatsDistVKDE(ng.StatsDistKernelST(16, 3.0), ng.StatsDistCV.NONE)
    sd.set_sample(g["centres"])
    sd.prepare()
    rng = np.random.default_rng(90001)
    for m in (90000, 262144):
        idx = rng.integers(0, g["centres"].shape[0], size=m)
        pts = g["centres"][idx] + 0.3 * rng.standard_normal((m, 16))
        x = torch.tensor(pts, dtype=torch.float64, device="cuda")
        ref = torch.empty(m, dtype=torch.float64, device="cuda")
        out = torch.empty(m, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.check(L.ncg_sd_eval_m2lnp_device(sd._h, C.c_void_p(x.data_ptr()), m, C.c_void_p(ref.data_ptr())),
                   "ncg_sd_eval_m2lnp_device")
        _lib.check(L.ncg_sd_eval_m2lnp_device_noalloc(sd._h, C.c_void_p(x.data_ptr()), m, C.c_void_p(out.data_ptr())),
                   "ncg_sd_eval_m2lnp_device_noalloc")
        sd.synchronize()
        assert rel_err(out.cpu().numpy(), ref.cpu().numpy()) < FP64_TOL, m
