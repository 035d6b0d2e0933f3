"""scft_diblock_density_noalloc: the propagator-density entry point for
callers that cannot allocate GPU memory (under another framework's pool
allocator, with a fixed memory budget, or unable to accept the device-wide
wait of cudaFree).

It is called through the C ABI with device buffers that the caller owns and
must agree with the allocating entry point scft_diblock_density within the
FP64 bar of the parity tests (1e-10 relative), on two calls in a row with
different problems, so the shared scratch array is seen to be reset between
calls.  Kept in a file of its own that pytest collects last.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-10


def load_golden(name):
    from ref_case import Case

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    return c, z


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def call_noalloc(S, torch, c, nD, smwa, smwb):
    lib = S.load()
    dev = torch.device("cuda:0")
    a = torch.from_numpy(np.ascontiguousarray(smwa).view(np.float64).ravel()).to(dev)
    b = torch.from_numpy(np.ascontiguousarray(smwb).view(np.float64).ravel()).to(dev)
    ra = torch.zeros_like(a)
    rb = torch.zeros_like(a)
    Q = torch.zeros(2, dtype=torch.float64, device=dev)
    nx = (ctypes.c_int * 3)(*c.Nx)
    L = (ctypes.c_double * 3)(*c.L)
    stream = torch.cuda.current_stream().cuda_stream
    code = lib.scft_diblock_density_noalloc(nx, L, c.Nda, c.Ndb, nD, a.data_ptr(), b.data_ptr(), ra.data_ptr(),
                                            rb.data_ptr(), Q.data_ptr(), stream)
    assert code == S.OK, lib.scft_last_error()
    torch.cuda.synchronize()
    shape = smwa.shape
    out_a = ra.cpu().numpy().view(np.complex128).reshape(shape)
    out_b = rb.cpu().numpy().view(np.complex128).reshape(shape)
    q = Q.cpu().numpy()
    return out_a, out_b, complex(q[0], q[1])


def test_noalloc_matches_allocating_entry_point_twice():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    for name in ("tiny_plate", "tiny_negab_oddN"):
        c, z = load_golden(name)
        with S.Context(S.params_from_case(c)) as ctx:
            nD = ctx.info(0)["nD"]
            ra_ref, rb_ref, Q_ref = ctx.diblock_density(0, z["smwa0"], z["smwb0"])
        ra, rb, Q = call_noalloc(S, torch, c, nD, z["smwa0"], z["smwb0"])
        assert abs(Q - Q_ref) <= RHO_TOL * abs(Q_ref), name
        assert rel(ra, ra_ref) < RHO_TOL, name
        assert rel(rb, rb_ref) < RHO_TOL, name
        # and the reference's own densities for the same smeared fields
        assert rel(ra, z["rhoda0"]) < RHO_TOL, name


def test_noalloc_single_block_and_narrow_columns():
    """The single-propagator path (Nda == N: one working array, q-dagger
    equal to q) on the reference's own fixture, and a grid whose nx = 12 is
    not a multiple of 16 (z-pass tiles of 4 columns), each against
    scft_diblock_density."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    c, z = load_golden("tiny_single_block")
    with S.Context(S.params_from_case(c)) as ctx:
        nD = ctx.info(0)["nD"]
        ra_ref, rb_ref, Q_ref = ctx.diblock_density(0, z["smwa0"], z["smwb0"])
    ra, rb, Q = call_noalloc(S, torch, c, nD, z["smwa0"], z["smwb0"])
    assert abs(Q - Q_ref) <= RHO_TOL * abs(Q_ref)
    assert rel(ra, ra_ref) < RHO_TOL
    assert rel(ra, z["rhoda0"]) < RHO_TOL

    from ref_case import Case

    c = Case(Nda=4, Ndb=3, Nx=(12, 6, 10), L=(3.0, 2.0, 2.5))
    rng = np.random.default_rng(31)
    wa = 0.3 * rng.standard_normal(c.shape) + 0j
    wb = 0.3 * rng.standard_normal(c.shape) + 0j
    with S.Context(S.params_from_case(c)) as ctx:
        nD = ctx.info(0)["nD"]
        ra_ref, rb_ref, Q_ref = ctx.diblock_density(0, wa, wb)
    for _ in range(2):
        ra, rb, Q = call_noalloc(S, torch, c, nD, wa, wb)
        assert abs(Q - Q_ref) <= RHO_TOL * abs(Q_ref)
        assert rel(ra, ra_ref) < RHO_TOL and rel(rb, rb_ref) < RHO_TOL


def test_noalloc_near_its_scratch_limit():
    """32^3 with N = 110 uses about 59 of the 64 MiB: it matches the
    allocating entry point; N = 130 at the same grid is rejected."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S
    from ref_case import Case

    c = Case(Nda=55, Ndb=55, Nx=(32, 32, 32), L=(10.0, 10.0, 10.0))
    rng = np.random.default_rng(37)
    wa = 0.05 * rng.standard_normal(c.shape) + 0j
    wb = 0.05 * rng.standard_normal(c.shape) + 0j
    with S.Context(S.params_from_case(c)) as ctx:
        nD = ctx.info(0)["nD"]
        ra_ref, rb_ref, Q_ref = ctx.diblock_density(0, wa, wb)
    ra, rb, Q = call_noalloc(S, torch, c, nD, wa, wb)
    assert abs(Q - Q_ref) <= RHO_TOL * abs(Q_ref)
    assert rel(ra, ra_ref) < RHO_TOL and rel(rb, rb_ref) < RHO_TOL
    lib = S.load()
    nx = (ctypes.c_int * 3)(32, 32, 32)
    L = (ctypes.c_double * 3)(10.0, 10.0, 10.0)
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda:0").data_ptr()
    assert lib.scft_diblock_density_noalloc(nx, L, 65, 65, 1.0, dummy, dummy, dummy, dummy, dummy, None) == S.ERR_ARG


def test_noalloc_rejects_problems_beyond_its_scratch():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    lib = S.load()
    nx = (ctypes.c_int * 3)(64, 64, 64)
    L = (ctypes.c_double * 3)(26.0, 26.0, 26.0)
    dummy = torch.zeros(2, dtype=torch.float64, device="cuda:0").data_ptr()
    code = lib.scft_diblock_density_noalloc(nx, L, 50, 50, 1.0, dummy, dummy, dummy, dummy, dummy, None)
    assert code == S.ERR_ARG
    assert b"64 MiB" in lib.scft_last_error()
