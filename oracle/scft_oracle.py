"""CPU restatement (numpy, FP64 complex) of the reference SCFT hot path.

TEST INFRASTRUCTURE ONLY.  tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use this module to check results against; the product (libscft) never
calls it.

Parity is pinned: tests/test_oracle.py runs this restatement against the
reference's own code compiled here (oracle/_ref/scft_ref, built by
oracle/Makefile) and against the committed fixtures in tests/golden/ that the
compiled reference produced (tests/golden/make_golden.py).

Layout: a grid array has numpy shape (Nz, Ny, Nx), x fastest, which is the
reference's stack order index = x + Nx*(y + Ny*z) (code/array_utils.cpp:80-87);
its FFTW plan runs on the reversed dimensions (code/array_utils.cpp:343-383),
i.e. an ordinary C-order 3-D DFT of this array.

Every function cites the reference file:line it restates.  All quantities are
in the reference's b-units.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.special import erfc

PI = 3.14159265358979323846263383  # code/globals.h:31


# --------------------------------------------------------------------------
# grid, FFT wrappers, integrals
# --------------------------------------------------------------------------
class Grid:
    """Grid bookkeeping of code/initialize.cpp:45-81 (M, V, dx)."""

    def __init__(self, Nx, L):
        self.Nx = tuple(int(n) for n in Nx)
        self.L = tuple(float(v) for v in L)
        self.dx = tuple(self.L[i] / self.Nx[i] for i in range(3))
        self.M = int(np.prod(self.Nx))
        self.V = float(np.prod(self.L))
        self.shape = (self.Nx[2], self.Nx[1], self.Nx[0])
        self.dV = self.dx[0] * self.dx[1] * self.dx[2]

    # code/array_utils.cpp:239-272 (get_k): k_i = 2*pi*n/L for n < N/2 else 2*pi*(n-N)/L
    def kvec_1d(self, d):
        n = np.arange(self.Nx[d], dtype=np.float64)
        return np.where(n < self.Nx[d] / 2.0, 2 * PI * n / self.L[d], 2 * PI * (n - self.Nx[d]) / self.L[d])

    def k_components(self):
        kx, ky, kz = self.kvec_1d(0), self.kvec_1d(1), self.kvec_1d(2)
        KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
        return KX, KY, KZ

    def k2(self):
        KX, KY, KZ = self.k_components()
        return KX * KX + KY * KY + KZ * KZ

    # code/array_utils.cpp:181-235 (get_k_alias): Nyquist components zeroed; any
    # point (other than the origin) with a zero component gets k = 0 entirely
    # when some axis has even length.
    def k_alias_components(self):
        comps = []
        for d in range(3):
            n = np.arange(self.Nx[d])
            k = self.kvec_1d(d).copy()
            if self.Nx[d] % 2 == 0:
                k[n == self.Nx[d] // 2] = 0.0
            comps.append(k)
        KZ, KY, KX = np.meshgrid(comps[2], comps[1], comps[0], indexing="ij")
        has_nyquist = any(n % 2 == 0 for n in self.Nx)
        if has_nyquist:
            kill = (KX == 0.0) | (KY == 0.0) | (KZ == 0.0)
            kill[0, 0, 0] = False  # id2 == 0 is exempt
            KX = np.where(kill, 0.0, KX)
            KY = np.where(kill, 0.0, KY)
            KZ = np.where(kill, 0.0, KZ)
        return KX, KY, KZ

    # code/array_utils.cpp:159-179 (get_r): minimum-image position
    def r_components(self):
        comps = []
        for d in range(3):
            r = self.dx[d] * np.arange(self.Nx[d], dtype=np.float64)
            r = np.where(r > self.L[d] / 2.0, r - self.L[d], r)
            r = np.where(r <= -self.L[d] / 2.0, r + self.L[d], r)
            comps.append(r)
        Z, Y, X = np.meshgrid(comps[2], comps[1], comps[0], indexing="ij")
        return X, Y, Z


def fft_fwd(g: Grid, a):
    """code/fft_wrappers.cpp:4-32: FFTW_FORWARD scaled by 1/M."""
    return np.fft.fftn(a) / g.M


def fft_bck(g: Grid, a):
    """code/fft_wrappers.cpp:35-64: FFTW_BACKWARD, unscaled."""
    return np.fft.ifftn(a) * g.M


def integ_trapPBC(g: Grid, f) -> complex:
    """code/integrate_utils.cpp:24-45: sum(f) * prod(dx)."""
    s = complex(np.sum(f))
    for d in range(3):
        s *= g.dx[d]
    return s


# --------------------------------------------------------------------------
# per-instance tables
# --------------------------------------------------------------------------
def hhat(g: Grid, a_smear: float):
    """code/initialize.cpp:97-102: exp(-k^2 a^2 / 2)."""
    return np.exp(-g.k2() * (a_smear * a_smear) / 2.0).astype(np.complex128)


def poly_bond_fft(g: Grid):
    """code/initialize.cpp:401-404: exp(-k^2/6) (bond length b = 1)."""
    return np.exp(-g.k2() / 6.0).astype(np.complex128)


def calc_gaa(g: Grid, fD: float, Rg2: float):
    """code/calc_debye.cpp:5-19."""
    k2 = g.k2() * Rg2
    with np.errstate(divide="ignore", invalid="ignore"):
        out = 2.0 * (np.exp(-k2 * fD) + fD * k2 - 1.0) / k2 / k2
    out.flat[0] = fD * fD
    return out.astype(np.complex128)


def calc_gbb(g: Grid, fD: float, Rg2: float):
    """code/calc_debye.cpp:21-35."""
    k2 = g.k2() * Rg2
    with np.errstate(divide="ignore", invalid="ignore"):
        out = 2.0 * (np.exp(-k2 * (1.0 - fD)) + (1.0 - fD) * k2 - 1.0) / k2 / k2
    out.flat[0] = (1.0 - fD) * (1.0 - fD)
    return out.astype(np.complex128)


def calc_gab(g: Grid, fD: float, Rg2: float):
    """code/calc_debye.cpp:37-51."""
    k2 = g.k2() * Rg2
    with np.errstate(divide="ignore", invalid="ignore"):
        out = (1.0 - np.exp(-k2 * fD)) * (1.0 - np.exp(-k2 * (1.0 - fD))) / k2 / k2
    out.flat[0] = fD * (1.0 - fD)
    return out.astype(np.complex128)


def calc_gd(g: Grid, alpha: float, Rg2: float):
    """code/calc_debye.cpp:53-68."""
    dm1 = g.k2() * Rg2 * alpha
    with np.errstate(divide="ignore", invalid="ignore"):
        out = np.where(dm1 == 0.0, 1.0, 2.0 * (np.exp(-dm1) + dm1 - 1.0) / dm1 / dm1)
    return out.astype(np.complex128)


def explicit_nanorod(g: Grid, length, rad, xi, rel_center, u):
    """code/initialize.cpp:578-612: 0.25*erfc((|u.r|-len/2)/xi)*erfc((|u x r|-rad)/xi)
    with r the minimum-image vector from the centre (code/array_utils.cpp:588-601)."""
    center = [rel_center[d] * g.L[d] for d in range(3)]
    comps = []
    for d in range(3):
        x = g.dx[d] * np.arange(g.Nx[d], dtype=np.float64)
        dr = x - center[d]
        dr = np.where(dr >= 0.5 * g.L[d], dr - g.L[d], np.where(dr < -0.5 * g.L[d], dr + g.L[d], dr))
        comps.append(dr)
    DZ, DY, DX = np.meshgrid(comps[2], comps[1], comps[0], indexing="ij")
    udr = u[0] * DX + u[1] * DY + u[2] * DZ
    c0 = u[1] * DZ - u[2] * DY
    c1 = u[2] * DX - u[0] * DZ
    c2 = u[0] * DY - u[1] * DX
    ucr = np.sqrt(c0 * c0 + c1 * c1 + c2 * c2)
    return (0.25 * erfc((np.abs(udr) - 0.5 * length) / xi) * erfc((np.abs(ucr) - rad) / xi)).astype(
        np.complex128)


def cuboid_frame(u):
    """In-plane axes of the cuboid plate (project extension, no reference
    counterpart): e1 = u x z normalised when |u_z| < 0.9, else u x x
    normalised; e2 = u x e1."""
    u = np.asarray(u, float)
    t = np.cross(u, (0.0, 0.0, 1.0)) if abs(u[2]) < 0.9 else np.cross(u, (1.0, 0.0, 0.0))
    e1 = t / np.linalg.norm(t)
    return e1, np.cross(u, e1)


def cuboid_plate(g: Grid, length, rad, xi, rel_center, u):
    """Project extension without a reference counterpart (SCFT_PLATE_CUBOID):
    a slab of thickness len along u and a 2 rad x 2 rad square in the plane,
    1/8 erfc((|u.r|-len/2)/xi) erfc((|e1.r|-rad)/xi) erfc((|e2.r|-rad)/xi),
    r the minimum-image vector from the centre as in explicit_nanorod."""
    center = [rel_center[d] * g.L[d] for d in range(3)]
    comps = []
    for d in range(3):
        dr = g.dx[d] * np.arange(g.Nx[d], dtype=np.float64) - center[d]
        comps.append(np.where(dr >= 0.5 * g.L[d], dr - g.L[d], np.where(dr < -0.5 * g.L[d], dr + g.L[d], dr)))
    DZ, DY, DX = np.meshgrid(comps[2], comps[1], comps[0], indexing="ij")
    e1, e2 = cuboid_frame(u)
    out = 0.125 * np.ones(DX.shape)
    for e, half in ((np.asarray(u, float), 0.5 * length), (e1, rad), (e2, rad)):
        p = e[0] * DX + e[1] * DY + e[2] * DZ
        out = out * erfc((np.abs(p) - half) / xi)
    return out.astype(np.complex128)


def field_gradient(g: Grid, a, d):
    """code/array_utils.cpp:565-579: spectral derivative with get_k_alias."""
    K = g.k_alias_components()[d]
    return fft_bck(g, fft_fwd(g, a) * (1j * K))


# --------------------------------------------------------------------------
# system setup (code/initialize.cpp:45-412) and state
# --------------------------------------------------------------------------
@dataclass
class System:
    """Parameters + derived tables of one SCFT instance (reference semantics)."""

    Nda: int
    Ndb: int
    a_smear: float
    rho0: float
    chi_ab: float  # signed, as in bcp.input
    chi_bc: float
    chi_ac: float
    kappa: float
    Nx: tuple
    L: tuple
    lam_pl: float
    lam_mi: float
    n_exp_nr: int = 0
    np_type: int = 2
    np_chem: int = 0
    sigma: float = 0.0
    Ng: int = 0
    L_nr: float = 1.0
    R_nr: float = 1.0
    xi_nr: float = 0.2
    centers: tuple = ((0.5, 0.5, 0.5), (0.5, 0.5, 0.5))
    orients: tuple = ((1.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    # project extension without a reference counterpart: potential lam on A
    # segments in the shell between the plate and the plate enlarged by w
    shell_lambda: float = 0.0
    shell_width: float = 0.0
    # project extension: 0 = the reference's disc, 1 = cuboid_plate
    plate_shape: int = 0
    update_scheme: int = 1  # bcp.input numbering: 0 = Euler, otherwise 1S (code/simulate.cpp:86-89)
    tables: dict = field(default_factory=dict)

    def __post_init__(self):
        # code/read_input.cpp:53-85: negative chi stored as |chi| with a flag
        self.neg_ab = int(self.chi_ab < 0)
        self.neg_bc = int(self.chi_bc < 0)
        self.neg_ac = int(self.chi_ac < 0)
        self.cab, self.cbc, self.cac = abs(self.chi_ab), abs(self.chi_bc), abs(self.chi_ac)
        if self.Ng == 0:
            self.sigma = 0.0  # code/read_input.cpp:200
        # code/read_input.cpp:220-235: orientation normalised as read
        self.orients = tuple(tuple(np.asarray(u, float) / max(np.linalg.norm(u), 1e-300)) for u in self.orients)
        self.g = Grid(self.Nx, self.L)
        self.initialize()

    @classmethod
    def from_case(cls, c) -> "System":
        return cls(Nda=c.Nda, Ndb=c.Ndb, a_smear=c.a_smear, rho0=c.rho0, chi_ab=c.chi_ab,
                   chi_bc=c.chi_bc, chi_ac=c.chi_ac, kappa=c.kappa, Nx=c.Nx, L=c.L,
                   lam_pl=c.lam_pl, lam_mi=c.lam_mi, n_exp_nr=c.n_exp_nr, np_type=c.np_type,
                   np_chem=c.np_chem, sigma=c.sigma, Ng=c.Ng, L_nr=c.L_nr, R_nr=c.R_nr,
                   xi_nr=c.xi_nr, centers=c.centers, orients=c.orients,
                   update_scheme=getattr(c, "update_scheme", 1))

    def plate(self, length, rad, i):
        shape = cuboid_plate if self.plate_shape == 1 else explicit_nanorod
        return shape(self.g, length, rad, self.xi_nr, self.centers[i], self.orients[i])

    def initialize(self):
        g = self.g
        self.N = self.Nda + self.Ndb  # code/initialize.cpp:53
        self.fD = self.Nda / self.N if self.N > 0 else 0.0
        self.Rg2 = (self.N - 1) / 6.0  # code/initialize.cpp:55
        t = self.tables
        t["hhat"] = hhat(g, self.a_smear)
        z = np.zeros(g.shape, np.complex128)
        rho_exp_nr = z.copy()
        expl_grafts = z.copy()
        if self.n_exp_nr > 0 and self.np_type != 2:
            raise NotImplementedError("only np_type=2 (nanorod/plate) explicit particles")
        # code/initialize.cpp:160-200: graft map = |grad rho_p(1.05 L, 1.05 R)|, normalised
        for i in range(self.n_exp_nr):
            pd = self.plate(self.L_nr * 1.05, self.R_nr * 1.05, i)
            grad2 = sum(field_gradient(g, pd, d) ** 2 for d in range(3))
            expl_grafts = expl_grafts + np.sqrt(grad2)
        if self.n_exp_nr > 0:
            expl_grafts = expl_grafts / integ_trapPBC(g, expl_grafts)
        # code/initialize.cpp:210-239: core density
        for i in range(self.n_exp_nr):
            rho_exp_nr = rho_exp_nr + self.plate(self.L_nr, self.R_nr, i)
        t["rho_exp_nr"] = rho_exp_nr
        t["exp_nrH"] = fft_fwd(g, rho_exp_nr)
        # extension: U_A = lam * sum_j [rho_p(L + 2w, R + w) - rho_p(L, R)]
        shellU = np.zeros(g.shape)
        if self.shell_lambda != 0.0:
            big = sum(self.plate(self.L_nr + 2 * self.shell_width, self.R_nr + self.shell_width, i)
                      for i in range(self.n_exp_nr))
            shellU = self.shell_lambda * (big.real - rho_exp_nr.real)
        t["shellU"] = shellU
        # code/initialize.cpp:249-386: volumes and chain counts (no film, no field NPs)
        V_exp = integ_trapPBC(g, rho_exp_nr).real
        self.Vf = g.V
        self.np_frac = V_exp / self.Vf
        V_1 = V_exp / self.n_exp_nr if self.n_exp_nr > 0 else 0.0
        if self.sigma > 0.0 and self.n_exp_nr > 0:
            expl_grafts = expl_grafts * (1.0 / integ_trapPBC(g, expl_grafts))  # :309-321
        t["expl_grafts"] = expl_grafts
        self.nP = 0.0 if self.n_exp_nr == 0 else V_exp / V_1
        if self.sigma > 0.0:
            self.ng_per_np = self.sigma * 4.0 * PI * self.R_nr * self.R_nr  # Dim == 3
            self.phiG = self.ng_per_np * self.nP * self.Ng / self.rho0 / self.Vf
        else:
            self.ng_per_np = 0.0
            self.phiG = 0.0
        self.phiD = 1.0 - 0.0 - self.np_frac - self.phiG  # phiH = 0
        self.nD = self.phiD * self.rho0 * self.Vf / self.N
        # Debye functions code/initialize.cpp:389-394
        t["gaa"] = calc_gaa(g, self.fD, self.Rg2)
        t["gbb"] = calc_gbb(g, self.fD, self.Rg2)
        t["gab"] = calc_gab(g, self.fD, self.Rg2)
        t["gc"] = calc_gd(g, (self.Ng - 1) / (self.N - 1), self.Rg2) if self.sigma > 0 else z.copy()
        t["gd"] = z.copy()
        t["poly_bond_fft"] = poly_bond_fft(g)


@dataclass
class State:
    wpl: np.ndarray
    wabp: np.ndarray
    wabm: np.ndarray
    wbcp: np.ndarray
    wbcm: np.ndarray
    wacp: np.ndarray
    wacm: np.ndarray
    out: dict = field(default_factory=dict)

    @classmethod
    def from_fields(cls, g: Grid, fields: dict) -> "State":
        z = np.zeros(g.shape, np.complex128)
        return cls(**{n: np.asarray(fields.get(n, z), np.complex128).reshape(g.shape).copy()
                      for n in ("wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm")})


# --------------------------------------------------------------------------
# propagators and densities
# --------------------------------------------------------------------------
def diblock_discrete(s: System, WA, WB, Ns=None, Na=None):
    """code/diblock_discrete.cpp:4-95.  Returns (Q, q, qdag), q/qdag of shape (Ns, ...)."""
    g = s.g
    Ns = s.N if Ns is None else Ns
    Na = s.Nda if Na is None else Na
    pb = s.tables["poly_bond_fft"]
    q = np.empty((Ns,) + g.shape, np.complex128)
    qd = np.empty_like(q)
    eA, eB = np.exp(-WA), np.exp(-WB)
    q[0] = eA if Na != 0 else eB
    qd[0] = eB if Na != s.N else eA
    for n in range(1, Ns):
        w = eA if (Na > 0 and n < Na) else eB
        q[n] = fft_bck(g, fft_fwd(g, q[n - 1]) * pb) * w
        if Na != Ns and Na != 0:
            w = eB if n <= (Ns - Na - 1) else eA
            qd[n] = fft_bck(g, fft_fwd(g, qd[n - 1]) * pb) * w
        else:
            qd[n] = q[n]
    Q = integ_trapPBC(g, q[s.N - 1]) / g.V
    return Q, q, qd


def integrate_diblock_discrete(s: System, q, qd, Q, nK, wA, wB, Ns=None, Na=None):
    """code/calc_poly_density.cpp:167-191."""
    Ns = s.N if Ns is None else Ns
    Na = s.Nda if Na is None else Na
    factor = nK / Q / s.g.V
    ra = np.zeros(s.g.shape, np.complex128)
    rb = np.zeros(s.g.shape, np.complex128)
    for j in range(Ns):
        term = q[j] * qd[Ns - j - 1]
        if Na > 0 and j < Na:
            ra += term
        else:
            rb += term
    ra *= np.exp(wA) * factor
    rb *= np.exp(wB) * factor
    return ra, rb


def homopolymer_discrete(s: System, WA, N):
    """code/homopolymer_discrete.cpp:3-55."""
    g = s.g
    pb = s.tables["poly_bond_fft"]
    q = np.empty((N,) + g.shape, np.complex128)
    e = np.exp(-WA)
    q[0] = e
    for n in range(1, N):
        q[n] = fft_bck(g, fft_fwd(g, q[n - 1]) * pb) * e
    return integ_trapPBC(g, q[N - 1]) / g.V, q


def integrate_homopoly_discrete(s: System, q, Q, nK, W, N):
    """code/calc_poly_density.cpp:193-212."""
    rh = np.zeros(s.g.shape, np.complex128)
    for j in range(N):
        rh += q[j] * q[N - j - 1]
    return rh * np.exp(W) * (nK / Q / s.g.V)


def graft_homopoly_free_ends(s: System, smwg, Ng):
    """code/grafted_nanoparticle.cpp:15-42."""
    g = s.g
    pb = s.tables["poly_bond_fft"]
    e = np.exp(-smwg)
    q = np.empty((Ng,) + g.shape, np.complex128)
    q[0] = e
    for j in range(1, Ng):
        q[j] = fft_bck(g, fft_fwd(g, q[j - 1]) * pb) * e
    return q


def grafted_exp_nps(s: System, smwg, qg):
    """code/grafted_nanoparticle.cpp:44-117.  Returns (Qga, qgdag, rhog)."""
    g = s.g
    Ng = s.Ng
    pb = s.tables["poly_bond_fft"]
    grafts = s.tables["expl_grafts"]
    e = np.exp(-smwg)
    qdg = np.empty_like(qg)
    qdg[0] = grafts * e / qg[Ng - 1]
    for j in range(1, Ng):
        qdg[j] = fft_bck(g, fft_fwd(g, qdg[j - 1]) * pb) * e
    rho = np.zeros(g.shape, np.complex128)
    for j in range(Ng):
        rho += qg[j] * qdg[Ng - j - 1]
    rho *= s.ng_per_np * s.n_exp_nr * np.exp(smwg)
    if np.any(qg[Ng - 1].real <= 0.0):
        raise FloatingPointError("non-positive graft propagator (code/grafted_nanoparticle.cpp:87-107)")
    tmp = np.where(grafts.real <= 0.0, 0.0, grafts * np.log(qg[Ng - 1]))
    return integ_trapPBC(g, tmp), qdg, rho


def assemble_fields(s: System, st: State):
    """code/calc_poly_density.cpp:42-64: w_A, w_B, w_G from the seven fields."""
    I = 1j
    wa = I * st.wpl + (I * st.wabm - st.wabp if s.neg_ab else I * st.wabp - st.wabm) \
        + (I * st.wacm - st.wacp if s.neg_ac else I * st.wacp - st.wacm)
    wb = I * st.wpl + (-I * st.wabm - st.wabp if s.neg_ab else I * st.wabp + st.wabm) \
        + (I * st.wbcm - st.wbcp if s.neg_bc else I * st.wbcp - st.wbcm)
    wg = I * st.wpl + (-I * st.wacm - st.wacp if s.neg_ac else I * st.wacp + st.wacm) \
        + (-I * st.wbcm - st.wbcp if s.neg_bc else I * st.wbcp + st.wbcm)
    return wa, wb, wg


def calc_poly_density(s: System, st: State, keep_hist=False):
    """code/calc_poly_density.cpp:37-161 (diblock + explicit grafted plates)."""
    g = s.g
    hh = s.tables["hhat"]
    wa, wb, wg = assemble_fields(s, st)
    smwa = fft_bck(g, fft_fwd(g, wa) * hh)
    smwb = fft_bck(g, fft_fwd(g, wb) * hh)
    smwg = fft_bck(g, fft_fwd(g, wg) * hh)
    o = st.out
    o.update(smwa=smwa, smwb=smwb, smwg=smwg)
    if s.nD > 0.0:
        ua = smwa + s.tables["shellU"]  # the extension's shell potential acts on A segments
        Qd, q, qd = diblock_discrete(s, ua, smwb)
        o["rhoda"], o["rhodb"] = integrate_diblock_discrete(s, q, qd, Qd, s.nD, ua, smwb)
        if keep_hist:
            o["qd"], o["qddag"] = q, qd
    else:
        Qd = 1.0
        o["rhoda"] = np.zeros(g.shape, np.complex128)
        o["rhodb"] = np.zeros(g.shape, np.complex128)
    o["Qd"] = Qd
    o.setdefault("rhog_exp", np.zeros(g.shape, np.complex128))
    o.setdefault("Qga", 0.0)
    if s.nP > 0.0 and s.sigma != 0:
        qg = graft_homopoly_free_ends(s, smwg, s.Ng)
        if s.n_exp_nr > 0 and s.sigma > 0.0:
            o["Qga"], qdg, o["rhog_exp"] = grafted_exp_nps(s, smwg, qg)
            if keep_hist:
                o["qg"], o["qgdag"] = qg, qdg
    return o


# --------------------------------------------------------------------------
# semi-implicit update and Hamiltonian
# --------------------------------------------------------------------------
def update_1s(s: System, st: State):
    """code/1s_update.cpp:7-352 (mean-field, no film/channel/field NPs)."""
    g = s.g
    I = 1j
    t = s.tables
    hh, gaa, gab, gbb, gc = t["hhat"], t["gaa"], t["gab"], t["gbb"], t["gc"]
    o = st.out
    rho0, N, Ng, phiD, phiG = s.rho0, s.N, s.Ng, s.phiD, s.phiG
    li, lr = s.lam_pl, s.lam_mi
    rhoda = fft_fwd(g, o["rhoda"]) if s.nD > 0.0 else o["rhoda"]
    rhodb = fft_fwd(g, o["rhodb"]) if s.nD > 0.0 else o["rhodb"]
    rhog_exp = o["rhog_exp"]
    if s.sigma > 0.0 and s.n_exp_nr > 0:
        rhog_exp = fft_fwd(g, rhog_exp)
    wpl = fft_fwd(g, st.wpl)
    if s.cab != 0.0:
        wabm, wabp = fft_fwd(g, st.wabm), fft_fwd(g, st.wabp)
    if s.cbc != 0.0:
        wbcm, wbcp = fft_fwd(g, st.wbcm), fft_fwd(g, st.wbcp)
    if s.cac != 0.0:
        wacm, wacp = fft_fwd(g, st.wacm), fft_fwd(g, st.wacp)
    z = np.zeros(g.shape, np.complex128)
    rhoha = z  # homopolymer and field NPs are absent
    surfH = z
    exp_nrH = t["exp_nrH"]
    evar = np.zeros(g.shape)
    evar.flat[0] = 1.0
    # w+ (:58-84)
    F = I * rho0 * (surfH + exp_nrH - evar) + I * 0.0 + I * hh * (rhoha + rhoda + t.get("rhog0", z) + rhog_exp + rhodb)
    A = (0.0 if s.kappa <= 0.0 else rho0 / s.kappa) + phiD * rho0 * N * hh * hh * (gaa + 2.0 * gab + gbb) \
        + (0.0 + phiG * Ng * gc) * rho0 * hh * hh
    if s.kappa > 0:
        B = A - rho0 / s.kappa
    else:
        raise NotImplementedError("kappa <= 0 leaves B uninitialised in code/1s_update.cpp:72-78")
    wpl = (wpl - li * (F - B * wpl)) / (1.0 + li * A)
    # AB (:87-166)
    if s.cab != 0.0:
        c = s.cab
        if not s.neg_ab:
            F = I * hh * (rhoda + rhodb + rhoha)
            if s.np_chem == 1:
                F = F - 0.0 - rho0 * exp_nrH
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * (gaa + 2.0 * gab + gbb)
            B = A - 2.0 * rho0 / c
            wabp = (wabp - li * (F - B * wabp)) / (1.0 + li * A)
            F = hh * (rhodb - rhoda - rhoha)
            if s.np_chem == 1:
                F = F + I * 0.0 + I * rho0 * exp_nrH
            wabm = (wabm - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
        else:
            F = -hh * (rhoda + rhodb + rhoha)
            wabp = (wabp - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
            F = I * hh * (rhoda - rhodb + rhoha)
            if s.np_chem == 1:
                F = F - 0.0 - rho0 * exp_nrH
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * (gaa - gbb)
            B = A - 2.0 * rho0 / c
            wabm = (wabm - li * (F - B * wabm)) / (1.0 + li * A)
    else:
        wabp = z.copy()
        wabm = z.copy()
    # BC (:168-247)
    if s.cbc != 0.0:
        c = s.cbc
        if not s.neg_bc:
            F = I * hh * (rhog_exp + rhodb)
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * (+gbb) + phiG * rho0 * Ng * hh * hh * gc
            B = A - 2.0 * rho0 / c
            wbcp = (wbcp - li * (F - B * wbcp)) / (1.0 + li * A)
            F = hh * (rhog_exp - rhodb)
            if s.np_chem == 1:
                F = F + I * 0.0 + I * rho0 * exp_nrH
            wbcm = (wbcm - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
        else:
            F = -hh * (rhodb + rhog_exp)
            wbcp = (wbcp - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
            F = -I * hh * (rhog_exp - rhodb)
            if s.np_chem == 1:
                F = F - 0.0 - rho0 * exp_nrH
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * gbb - phiG * Ng * hh * hh * rho0 * gc
            B = A - 2.0 * rho0 / c
            wbcm = (wbcm - li * (F - B * wbcm)) / (1.0 + li * A)
    else:
        wbcp = z.copy()
        wbcm = z.copy()
    # AC (:250-329)
    if s.cac != 0.0:
        c = s.cac
        if not s.neg_ac:
            F = I * hh * (rhog_exp + rhoda)
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * gaa + phiG * Ng * hh * hh * rho0 * gc
            B = A - 2.0 * rho0 / c
            wacp = (wacp - li * (F - B * wacp)) / (1.0 + li * A)
            F = hh * (rhog_exp - rhoda)
            if s.np_chem == 1:
                F = F + I * 0.0 + I * rho0 * exp_nrH
            wacm = (wacm - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
        else:
            F = -hh * (rhoda + rhog_exp)
            wacp = (wacp - lr * F) / (1.0 + lr * 2.0 * rho0 / c)
            F = -I * hh * (rhog_exp - rhoda)
            if s.np_chem == 1:
                F = F - 0.0 - rho0 * exp_nrH
            A = 2.0 * rho0 / c + phiD * rho0 * N * hh * hh * gaa - phiG * Ng * hh * hh * rho0 * gc
            B = A - 2.0 * rho0 / c
            wacm = (wacm - li * (F - B * wacm)) / (1.0 + li * A)
    else:
        wacp = z.copy()
        wacm = z.copy()
    # back to real space (:331-349)
    st.wpl = fft_bck(g, wpl)
    st.wabm, st.wabp = (fft_bck(g, wabm), fft_bck(g, wabp)) if s.cab != 0.0 else (wabm, wabp)
    st.wbcm, st.wbcp = (fft_bck(g, wbcm), fft_bck(g, wbcp)) if s.cbc != 0.0 else (wbcm, wbcp)
    st.wacm, st.wacp = (fft_bck(g, wacm), fft_bck(g, wacp)) if s.cac != 0.0 else (wacm, wacp)
    return calc_poly_density(s, st)


def update_euler(s: System, st: State):
    """code/Euler_update.cpp:5-213 (mean field: no noise, homopolymer, field
    NPs, channel or film): w <- w - lam dH/dw in k-space, lam_pl for w+ and
    the + fields, lam_mi for the - fields."""
    g = s.g
    I = 1j
    t = s.tables
    hh = t["hhat"]
    o = st.out
    rho0, li, lr = s.rho0, s.lam_pl, s.lam_mi
    z = np.zeros(g.shape, np.complex128)
    rhoda = fft_fwd(g, o["rhoda"]) if s.nD > 0.0 else o["rhoda"]
    rhodb = fft_fwd(g, o["rhodb"]) if s.nD > 0.0 else o["rhodb"]
    rhog_exp = fft_fwd(g, o["rhog_exp"]) if (s.sigma > 0.0 and s.n_exp_nr > 0) else o["rhog_exp"]
    evar = np.zeros(g.shape)
    evar.flat[0] = 1.0
    wpl = fft_fwd(g, st.wpl)
    F = (0.0 if s.kappa <= 0.0 else rho0 * wpl / s.kappa) + I * rho0 * (t["exp_nrH"] - evar) \
        + I * hh * (rhoda + rhodb + rhog_exp)
    st.wpl = fft_bck(g, wpl - li * F)

    def pair(c, neg, wp, wm, X, Y):
        if c == 0.0:
            return z.copy(), z.copy()
        wp, wm = fft_fwd(g, wp), fft_fwd(g, wm)
        Fp = 2.0 * rho0 * wp / c + hh * (X * (-1 if neg else I) + Y * (-1 if neg else I))
        Fm = 2.0 * rho0 * wm / c + hh * (X * (I if neg else -1) + Y * (-I if neg else 1))
        return fft_bck(g, wp - li * Fp), fft_bck(g, wm - lr * Fm)

    st.wabp, st.wabm = pair(s.cab, s.neg_ab, st.wabp, st.wabm, rhoda, rhodb)
    st.wbcp, st.wbcm = pair(s.cbc, s.neg_bc, st.wbcp, st.wbcm, rhodb, rhog_exp)
    st.wacp, st.wacm = pair(s.cac, s.neg_ac, st.wacp, st.wacm, rhoda, rhog_exp)
    return calc_poly_density(s, st)


def calc_H(s: System, st: State) -> complex:
    """code/calc_h.cpp:9-132."""
    g = s.g
    o = st.out
    rho_np = s.tables["rho_exp_nr"]
    tmp2 = (0.0 if s.kappa <= 0.0 else st.wpl * st.wpl * s.rho0 / s.kappa / 2.0) \
        - 1j * s.rho0 * (1.0 - 0.0 - rho_np) * st.wpl
    H = integ_trapPBC(g, tmp2)
    for c, neg, p, m in ((s.cbc, s.neg_bc, st.wbcp, st.wbcm), (s.cac, s.neg_ac, st.wacp, st.wacm),
                         (s.cab, s.neg_ab, st.wabp, st.wabm)):
        if c != 0.0:
            H += integ_trapPBC(g, (p * p + m * m) * s.rho0 / c * (-1.0 if neg else 1.0))
    if s.nD > 0.0:
        H += -s.nD * np.log(complex(o["Qd"]))
    if s.n_exp_nr > 0 and s.sigma > 0.0:
        H += -float(s.n_exp_nr) * s.ng_per_np * complex(o["Qga"]).real
    if H != H:
        raise FloatingPointError("H is NaN (code/calc_h.cpp:37-61)")
    return H


def run(s: System, st: State, iters: int):
    """code/simulate.cpp:36,74,85-99 with calc_H after every update: returns the
    trace rows [iter, Re H, Im H, Re Qd, Im Qd, Re Qga, Im Qga]."""
    calc_poly_density(s, st)
    rows = []

    def row(it):
        H = calc_H(s, st)
        Qd = complex(st.out["Qd"])
        Qga = complex(st.out["Qga"])
        rows.append([it, H.real, H.imag, Qd.real, Qd.imag, Qga.real, Qga.imag])

    row(0)
    step = update_euler if s.update_scheme == 0 else update_1s
    for it in range(1, iters + 1):
        step(s, st)
        row(it)
    return np.array(rows)


def converged_error(H_now: complex, H_prev: complex, V: float, print_freq: int) -> float:
    """code/simulate.cpp:112: err = |H - H_old| / V / print_freq."""
    return abs(H_now - H_prev) / V / float(print_freq)
