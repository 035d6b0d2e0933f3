"""scft_step_fields: one call that uploads the fields of every instance from
host memory, builds their densities, runs n_iter updates and returns H.  It
must give exactly what the call sequence scft_set_fields_all,
scft_update_1s, scft_calc_H gives (the same kernels on the same data; the
mixed form runs each sweep group's chain on its own stream in one captured
graph), on the first call (capture) and on replays with the same host
buffers, for the mixed form and for the FP64 method (which runs the
sequence).  Complex fields in the mixed form return SCFT_ERR_COMPLEX.

scft_iterate_fields: one iteration of the reference's main loop from and to
host memory (density build, H of the fields passed in, one update, the
updated fields written back).  Repeated calls on the same host buffers must
follow the device-resident sequence calc_H, update_1s: H of the first call
exactly (same kernels on the same data), later calls within 1e-9 of H (the
mixed form's fields pass through FP64 transforms on the way out and back in,
a 1e-16 relative change), the fields written back within 1e-11 of the
largest; the FP64 method exactly.  Without the download the context holds
the updated fields; pageable buffers take the call sequence and give the
same results; pairs whose chi is 0 enter with the caller's values and are
left as they were.
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


def arrays(S, ps, bufs):
    """complex128 views (7,) + grid of pinned buffers (or plain copies)."""
    return [b.t.numpy().view(np.complex128).reshape((7, p.Nx[2], p.Nx[1], p.Nx[0])) for p, b in zip(ps, bufs)]


def resident_trajectory(S, ps, fields, iters):
    """calc_H then update_1s, `iters` times, on the device; H of each
    iteration's fields and the fields after the last update."""
    Hs = []
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        for _ in range(iters):
            Hs.append(c.calc_H().copy())
            c.update_1s(1)
        w = [c.get_fields(k) for k in range(len(ps))]
        H_after = c.calc_H().copy()
    return Hs, w, H_after


def in_use(p):
    """Fields an update changes (w+ and the pairs of nonzero chi)."""
    return ["wpl"] + (["wabp", "wabm"] if p.chi_ab else []) + (["wbcp", "wbcm"] if p.chi_bc else []) + \
        (["wacp", "wacm"] if p.chi_ac else [])


@pytest.mark.parametrize("prec", [1, 0])
def test_iterate_fields_follows_the_resident_iteration(S, prec):
    ps, fields = batch(S, prec)
    Hs, w_ref, _ = resident_trajectory(S, ps, fields, 3)
    bufs = host_buffers(S, ps, fields)
    arrs = arrays(S, ps, bufs)
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        for it in range(3):  # capture, then replays on the same buffers
            H = c.iterate_fields(arrs)
            assert c.last_status == S.OK
            if it == 0 or prec == S.PREC_FP64:
                np.testing.assert_array_equal(H, Hs[it])
            else:
                assert np.abs(H[:, :4] - Hs[it][:, :4]).max() <= 1e-9 * np.abs(Hs[it][:, :4]).max()
    for p, a, wr in zip(ps, arrs, w_ref):
        for q, name in enumerate(S.FIELD_NAMES):
            if name in in_use(p) or prec == S.PREC_FP64:
                scale = max(np.abs(wr[name]).max(), 1e-300)
                assert np.abs(a[q] - wr[name]).max() <= (0.0 if prec == S.PREC_FP64 else 1e-11) * scale, name


def test_iterate_fields_without_download_leaves_the_updated_fields(S):
    ps, fields = batch(S, S.PREC_MIXED)
    Hs, w_ref, H_after = resident_trajectory(S, ps, fields, 1)
    bufs = host_buffers(S, ps, fields)
    arrs = arrays(S, ps, bufs)
    before = [a.copy() for a in arrs]
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        H = c.iterate_fields(arrs, download=False)
        np.testing.assert_array_equal(H, Hs[0])
        for a, b in zip(arrs, before):
            np.testing.assert_array_equal(a, b)
        for k, p in enumerate(ps):
            f = c.get_fields(k)
            for name in in_use(p):
                np.testing.assert_array_equal(f[name], w_ref[k][name])
        # the densities of the updated fields are rebuilt on demand
        H1 = c.calc_H()
        assert np.abs(H1[:, :4] - H_after[:, :4]).max() <= 1e-10 * np.abs(H_after[:, :4]).max()


def test_iterate_fields_from_pageable_buffers_takes_the_sequence(S):
    """Plain numpy arrays are not page-locked: the call runs the sequence
    and gives the graph's results; the pairs whose chi is 0 (given nonzero
    values here) keep the values the caller put there."""
    ps, fields = batch(S, S.PREC_MIXED)
    rng = np.random.default_rng(6)
    plain = []
    for p, f in zip(ps, fields):
        b = np.zeros((7, p.Nx[2], p.Nx[1], p.Nx[0]), np.complex128)
        for q, name in enumerate(S.FIELD_NAMES):
            b[q] = f.get(name, 0.0) if name in in_use(p) else 0.05 * rng.standard_normal(b.shape[1:])
        plain.append(b)
    junk = [b.copy() for b in plain]
    pb = host_buffers(S, ps, [{n: b[q] for q, n in enumerate(S.FIELD_NAMES)} for b in plain])
    pinned = arrays(S, ps, pb)
    res = []
    for arrs in (pinned, plain):
        with S.Context(ps) as c:
            c.set_sweep_groups(2)
            res.append([c.iterate_fields(arrs) for _ in range(2)])
    for a, b in zip(res[0], res[1]):
        assert np.abs(a[:, :4] - b[:, :4]).max() <= 1e-9 * np.abs(b[:, :4]).max()
    for p, x, y, j in zip(ps, pinned, plain, junk):
        for q, name in enumerate(S.FIELD_NAMES):
            if name in in_use(p):
                assert np.abs(x[q] - y[q]).max() <= 1e-11 * np.abs(y[q]).max(), name
            else:
                np.testing.assert_array_equal(x[q], j[q])
                np.testing.assert_array_equal(y[q], j[q])


def test_iterate_fields_rejects_complex_fields_in_the_mixed_form(S):
    ps, fields = batch(S, S.PREC_MIXED)
    fields[2] = dict(fields[2])
    fields[2]["wabm"] = fields[2]["wabm"] + 0.2j
    bufs = host_buffers(S, ps, fields)
    arrs = arrays(S, ps, bufs)
    with S.Context(ps) as c:
        with pytest.raises(S.ScftError) as e:
            c.iterate_fields(arrs)
        assert e.value.code == S.ERR_COMPLEX and "instance 2" in str(e.value)


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
    """The mixed form holds the pairs whose chi is 0 (here chi_bc = chi_ac =
    0) at zero, as the reference initialises them (its update never changes
    them, and the mixed update assembles w_A, w_B without them): values the
    caller puts there change nothing, through the call or through the
    sequence, and the context reads them back as zero."""
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
    with S.Context(ps) as c:
        c.set_sweep_groups(2)
        c.set_fields_all_raw([b.ctypes.data for b in dirty])
        assert np.abs(c.get_fields(1)["wbcp"]).max() == 0.0
        c.update_1s(1)
        res.append(c.calc_H().copy())
    np.testing.assert_array_equal(res[0], res[1])
    np.testing.assert_array_equal(res[0], res[2])
