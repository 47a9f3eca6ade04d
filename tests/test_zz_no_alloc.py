"""The zero-allocation two-axis transform against the workspace entry point.

pgx_cheb_transform_2d_noalloc serves callers that cannot let a library
allocate device memory (codes that own all device memory through their own
pool or budget, or time loops that must not pay cudaMalloc's implicit
synchronisation): its scratch and twiddle tables are static device arrays.
Its results must match pgx_cheb_transform_2d (caller workspace) to the
path's 1e-10 relative tolerance, call after call.  This file is collected
last so that a run stopping at the first failure has run every other test.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def env():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    from pypde_gb300 import _lib
    return torch, _lib


def run_pair(env, x, n_out, N, mode):
    """Same transform through both entry points; returns (workspace result, no-alloc result)."""
    torch, _lib = env
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    n0_in, n1_in = x.shape
    ref = torch.empty(n_out, dtype=torch.float64, device="cuda")
    got = torch.full(n_out, float("nan"), dtype=torch.float64, device="cuda")
    work = torch.empty(n_out[0] * n1_in, dtype=torch.float64, device="cuda")
    _lib.check(L.pgx_cheb_transform_2d(x.data_ptr(), n1_in, 1, n0_in, n1_in, ref.data_ptr(), n_out[1], 1,
                                       n_out[0], n_out[1], N[0], N[1], mode, work.data_ptr(), work.numel(), st),
               "pgx_cheb_transform_2d")
    _lib.check(L.pgx_cheb_transform_2d_noalloc(x.data_ptr(), n1_in, 1, n0_in, n1_in, got.data_ptr(), n_out[1], 1,
                                               n_out[0], n_out[1], N[0], N[1], mode, st),
               "pgx_cheb_transform_2d_noalloc")
    torch.cuda.synchronize()
    return ref.cpu().numpy(), got.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_twice(env):
    torch, _lib = env
    rng = np.random.default_rng(21)
    # call 1: dealiased backward of a 65 x 33 coefficient field onto the 97 x 49 grid
    c = torch.as_tensor(rng.uniform(-1, 1, (65, 33)), device="cuda")
    ref, got = run_pair(env, c, (97, 49), (97, 49), _lib.DCT_BWD)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) < TOL
    # call 2 right after, different shape and direction: dealiased forward 193 x 97 -> 129 x 65
    v = torch.as_tensor(rng.uniform(-1, 1, (193, 97)), device="cuda")
    ref, got = run_pair(env, v, (129, 65), (193, 97), _lib.DCT_FWD)
    assert np.isfinite(got).all()
    assert rel_err(got, ref) < TOL


def test_noalloc_rejects_sizes_beyond_its_static_scratch(env):
    torch, _lib = env
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    # n0_out * n1_in = 2049 * 1025 doubles exceeds PGX_NOALLOC_SCRATCH_DOUBLES: rejected before any launch
    assert L.pgx_cheb_transform_2d_noalloc(x.data_ptr(), 1025, 1, 2049, 1025, x.data_ptr(), 1025, 1, 2049, 1025,
                                           2049, 1025, _lib.DCT_BWD, st) == 1
    # a length without an FFT plan (the dense fallback would need an N x N table) is rejected too
    assert L.pgx_cheb_transform_2d_noalloc(x.data_ptr(), 40, 1, 40, 40, x.data_ptr(), 40, 1, 40, 40, 40, 40,
                                           _lib.DCT_BWD, st) == 1
