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
