"""The zero-allocation two-axis transform against the oracle and the workspace entry point.

pgx_cheb_transform_2d_noalloc serves callers that cannot let a library
allocate device memory (codes that own all device memory through their own
pool or budget, or time loops that must not pay cudaMalloc's implicit
synchronisation): its scratch and twiddle tables are static device arrays.

Each case calls the no-alloc entry point FIRST, on lengths that no other test
transforms (so the library's twiddle caches hold nothing for them and any
fallback to an allocating table would be the only way to get one), checks the
result against the CPU oracle's Chebyshev transforms, and only then runs the
workspace entry point pgx_cheb_transform_2d on the same input and checks that
both agree -- all to the path's 1e-10 relative tolerance, call after call.
This file is collected last so that a run stopping at the first failure has
run every other test.
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


def oracle_2d(x, n_out, N, forward):
    """The oracle's two-axis transform: axis 0 then axis 1, zero-padded to N before a backward
    transform (bases/utils.py:88-109), truncated to n_out after a forward one (utils.py:112-115)."""
    from oracle import spectral as sp
    from oracle.field import zero_pad, zero_unpad
    v = np.asarray(x, dtype=np.float64)
    for axis in (0, 1):
        if forward:
            v = zero_unpad(sp.cheb_forward(v, axis), n_out[axis], axis)
        else:
            v = sp.cheb_backward(zero_pad(v, N[axis], axis), axis)
            v = zero_unpad(v, n_out[axis], axis)
    return v


def no_alloc_then_workspace(env, x, n_out, N, mode):
    """The no-alloc call first, then the workspace call on the same input; returns both results."""
    torch, _lib = env
    L = _lib.lib()
    st = torch.cuda.current_stream().cuda_stream
    n0_in, n1_in = x.shape
    got = torch.full(n_out, float("nan"), dtype=torch.float64, device="cuda")
    _lib.check(L.pgx_cheb_transform_2d_noalloc(x.data_ptr(), n1_in, 1, n0_in, n1_in, got.data_ptr(), n_out[1], 1,
                                               n_out[0], n_out[1], N[0], N[1], mode, st),
               "pgx_cheb_transform_2d_noalloc")
    torch.cuda.synchronize()
    got_h = got.cpu().numpy()
    ref = torch.full(n_out, float("nan"), dtype=torch.float64, device="cuda")
    work = torch.empty(n_out[0] * n1_in, dtype=torch.float64, device="cuda")
    _lib.check(L.pgx_cheb_transform_2d(x.data_ptr(), n1_in, 1, n0_in, n1_in, ref.data_ptr(), n_out[1], 1,
                                       n_out[0], n_out[1], N[0], N[1], mode, work.data_ptr(), work.numel(), st),
               "pgx_cheb_transform_2d")
    torch.cuda.synchronize()
    return got_h, ref.cpu().numpy()


def test_noalloc_matches_oracle_and_workspace_entry_point_twice(env):
    torch, _lib = env
    rng = np.random.default_rng(21)
    # call 1: dealiased backward of a 55 x 19 coefficient field onto the 82 x 28 grid
    # (82 - 1 = 3^4, 28 - 1 = 3^3: FFT lengths no other test transforms)
    c = rng.uniform(-1, 1, (55, 19))
    got, ref = no_alloc_then_workspace(env, torch.as_tensor(c, device="cuda"), (82, 28), (82, 28), _lib.DCT_BWD)
    assert np.isfinite(got).all()
    assert rel_err(got, oracle_2d(c, (82, 28), (82, 28), forward=False)) < TOL
    assert rel_err(got, ref) < TOL
    # call 2 right after, other shape and direction: dealiased forward 163 x 55 -> 109 x 37
    # (163 - 1 = 2 * 3^4, 55 - 1 = 2 * 3^3); the static scratch still holds call 1's data
    v = rng.uniform(-1, 1, (163, 55))
    got, ref = no_alloc_then_workspace(env, torch.as_tensor(v, device="cuda"), (109, 37), (163, 55), _lib.DCT_FWD)
    assert np.isfinite(got).all()
    assert rel_err(got, oracle_2d(v, (109, 37), (163, 55), forward=True)) < TOL
    assert rel_err(got, ref) < TOL


def test_noalloc_two_point_lengths(env):
    """N = 2 (the smallest length the workspace entry point takes) on one axis, both directions."""
    torch, _lib = env
    rng = np.random.default_rng(22)
    c = rng.uniform(-1, 1, (2, 37))
    got, ref = no_alloc_then_workspace(env, torch.as_tensor(c, device="cuda"), (2, 37), (2, 37), _lib.DCT_BWD)
    assert rel_err(got, oracle_2d(c, (2, 37), (2, 37), forward=False)) < TOL
    assert rel_err(got, ref) < TOL
    got, ref = no_alloc_then_workspace(env, torch.as_tensor(c, device="cuda"), (2, 37), (2, 37), _lib.DCT_FWD)
    assert rel_err(got, oracle_2d(c, (2, 37), (2, 37), forward=True)) < TOL
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
    # and so is a one-point length
    assert L.pgx_cheb_transform_2d_noalloc(x.data_ptr(), 1, 1, 1, 1, x.data_ptr(), 1, 1, 1, 1, 1, 1,
                                           _lib.DCT_BWD, st) == 1
