"""scft_step_fields: one call that uploads the fields of every instance from
host memory, builds their densities, runs n_iter updates and returns H.  It
must give exactly what the call sequence scft_set_fields_all,
scft_update_1s, scft_calc_H gives (the same kernels on the same data; the
mixed form runs each sweep group's chain on its own stream in one captured
graph), on the first call (capture) and on replays with the same host
buffers, for the mixed form and for the FP64 method (which runs the
sequence).  Complex fields in the mixed form return SCFT_ERR_COMPLEX.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def batch(S, prec):
    from scft.workloads import plate_params, seeded_fields

    grids = [(64, 64, 64), (64, 64, 64), (48, 48, 48), (64, 64, 64)]
    ps = [plate_params(12.0 * k, N=10 + 2 * k, grid=g, box_rg=tuple(6.4 * n / 64 for n in g), precision=prec)
          for k, g in enumerate(grids)]
    return ps, [seeded_fields(p, 90 + k) for k, p in enumerate(ps)]


class Pinned:
    """A page-locked host copy of one instance's seven fields (torch pinned
    memory) and its address."""

    def __init__(self, S, p, f):
        import torch

        sh = (p.Nx[2], p.Nx[1], p.Nx[0])
        b = np.zeros((7,) + sh, np.complex128)
        for q, name in enumerate(S.FIELD_NAMES):
            if name in f:
                b[q] = f[name]
        self.t = torch.zeros(b.size * 2, dtype=torch.float64, pin_memory=True)
        self.t.numpy()[:] = b.view(np.float64).ravel()
        self.ctypes = type("P", (), {"data": self.t.data_ptr()})()


def host_buffers(S, ps, fields):
    return [Pinned(S, p, f) for p, f in zip(ps, fields)]


@pytest.mark.parametrize("prec", [1, 0])
def test_step_fields_matches_the_call_sequence(S, prec):
    ps, fields = batch(S, prec)
    bufs = host_buffers(S, ps, fields)
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        c.set_fields_all_raw([b.ctypes.data for b in bufs])
        c.update_1s(2)
        H_ref = c.calc_H().copy()
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        c.update_1s(1)  # the context has run before, as in a real loop
        out = np.zeros((len(ps), 5))
        for _ in range(3):  # capture, then replays with the same buffers
            out[:] = 0.0
            st = c.step_fields_raw([b.ctypes.data for b in bufs], 2, out.ctypes.data)
            assert st == S.OK
            np.testing.assert_array_equal(out, H_ref)


def test_step_fields_rejects_complex_fields_in_the_mixed_form(S):
    ps, fields = batch(S, S.PREC_MIXED)
    fields[1] = dict(fields[1])
    fields[1]["wabm"] = fields[1]["wabm"] + 0.3j
    bufs = host_buffers(S, ps, fields)
    with S.Context(ps) as c:
        out = np.zeros((len(ps), 5))
        with pytest.raises(S.ScftError) as e:
            c.step_fields_raw([b.ctypes.data for b in bufs], 1, out.ctypes.data)
        assert e.value.code == S.ERR_COMPLEX and "instance 1" in str(e.value)


def test_step_fields_ignores_the_pairs_whose_chi_is_zero(S):
    """Only w+ and the pairs of nonzero chi are read from the host: values in
    the others (here chi_bc = chi_ac = 0) change nothing."""
    ps, fields = batch(S, S.PREC_MIXED)
    rng = np.random.default_rng(5)
    noisy = []
    for p, f in zip(ps, fields):
        g = dict(f)
        sh = (p.Nx[2], p.Nx[1], p.Nx[0])
        for name in ("wbcp", "wbcm", "wacp", "wacm"):
            g[name] = rng.standard_normal(sh) + 0j
        noisy.append(g)
    clean, dirty = host_buffers(S, ps, fields), host_buffers(S, ps, noisy)
    res = []
    for bufs in (clean, dirty):
        with S.Context(ps) as c:
            c.set_sweep_groups(2)
            out = np.zeros((len(ps), 5))
            assert c.step_fields_raw([b.ctypes.data for b in bufs], 1, out.ctypes.data) == S.OK
            res.append(out.copy())
    np.testing.assert_array_equal(res[0], res[1])
