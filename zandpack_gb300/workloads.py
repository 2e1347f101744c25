"""Synthetic AME workloads in the reference's ``Arrays/`` format.

The reference builds its propagation inputs from DFT/TBtrans data through
``TD_Transport`` (Zandpack/TimedependentTransport.py:858-1038) and writes them
with ``Writer.write_to_file_compressed`` (Zandpack/Writer.py:61-151).  No such
data exists here, so this module restates that arithmetic on seeded
tight-binding models:

* lead level widths are sums of Lorentzians, Gamma_a(E) = sum_x G_x W_x^2 /
  ((E - e_x)^2 + W_x^2) with PSD coefficient matrices G_x on the lead's
  coupling orbitals (Zandpack/basicbackground.txt:17);
* ``GG_P, GL_P, GG_M, GL_M, Xpp, Xpm`` follow ``get_propagation_quantities``
  (Zandpack/TimedependentTransport.py:932-1038): Lorentzian modes from the
  eigenpairs of G_x, Fermi-pole modes from the Hermitian parts of Gamma_a at the
  Pade poles (``diagonalise``, :858-930), eigenvalues sorted by decreasing |l|;
* ``xi`` holds the eigenvectors embedded into the device basis, ``Ixi = conj(xi)``
  (:1027-1033); the eigen axis is written truncated to ``NOT`` because ``zand``
  only reads ``[..., :NOT]`` (Zandpack/mpi/zand:568-576);
* ``DM_Ortho`` is the isolated-device Fermi density matrix (the reference's
  default start, Zandpack/TimedependentTransport.py:1178-1187) and psi = Omega = 0.

Eigenvalues below ``1e-12 * max|l|`` are set to exactly zero, so rank-deficient
coefficient matrices give exactly-zero rows, as a rank-r fit means.

Every configuration is seeded with ``numpy.random.default_rng(1000 + k)``.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Callable, Optional

import numpy as np

from .constants import HBAR
from .pade import psd_poles, fermi_expanded

__all__ = ["Workload", "make_workload", "make_nonorth_workload", "make_kpoint_workload", "CONFIGS", "bias_value"]


# ---------------------------------------------------------------- lattices
def chain(n: int, t: float) -> np.ndarray:
    H = np.diag(np.full(n - 1, t), 1)
    return H + H.T


def square_lattice(nx: int, ny: int, t: float) -> np.ndarray:
    """Sites (i, j) -> i*ny + j; i is the transport (column) index."""
    n = nx * ny
    H = np.zeros((n, n))
    for i in range(nx):
        for j in range(ny):
            s = i * ny + j
            if i + 1 < nx:
                H[s, s + ny] = H[s + ny, s] = t
            if j + 1 < ny:
                H[s, s + 1] = H[s + 1, s] = t
    return H


def honeycomb_ribbon(ncol: int, nrow: int, t: float) -> np.ndarray:
    """Brick-wall honeycomb: sites (i, j) -> i*nrow + j with i the column.
    Bonds along a column always, across columns when (i + j) is even."""
    n = ncol * nrow
    H = np.zeros((n, n))
    for i in range(ncol):
        for j in range(nrow):
            s = i * nrow + j
            if j + 1 < nrow:
                H[s, s + 1] = H[s + 1, s] = t
            if i + 1 < ncol and (i + j) % 2 == 0:
                H[s, s + nrow] = H[s + nrow, s] = t
    return H


def random_sparse(n: int, rng, tmin: float, tmax: float) -> np.ndarray:
    """Degree-4 random graph: a ring plus a ring over a random permutation."""
    H = np.zeros((n, n))
    edges = set()
    for i in range(n):
        edges.add((min(i, (i + 1) % n), max(i, (i + 1) % n)))
    while True:
        p = rng.permutation(n)
        extra = {(min(p[i], p[(i + 1) % n]), max(p[i], p[(i + 1) % n])) for i in range(n)}
        if not (extra & edges):
            break
    for (a, b) in sorted(edges | extra):
        H[a, b] = H[b, a] = -rng.uniform(tmin, tmax)
    return H


# ---------------------------------------------------------------- workload
@dataclasses.dataclass
class Workload:
    """One propagation problem: the ``Arrays`` dictionary plus the run
    parameters an ``Initial.py``/``Bias.py`` pair would hold."""
    name: str
    arrays: dict
    t0: float
    t1: float
    eps: float
    stepsize: float
    hbar: float
    bias: dict                 # {"kind": ..., params}
    hubbard_U: Optional[float]  # dH(t, sig) = U * diag(Re diag sig - 0.5) when set
    kT: float
    coupling: list             # per lead: orbital indices

    @property
    def n(self) -> int:
        return self.arrays["H_Ortho"].shape[-1]

    @property
    def n_leads(self) -> int:
        return int(self.arrays["psi_shape"][1])

    def bias_fn(self) -> Callable[[float, int], float]:
        spec = dict(self.bias)
        return lambda t, a: bias_value(spec, t, a)

    def dH_fn(self) -> Callable:
        U = self.hubbard_U
        if U is None:
            return lambda t, sig: 0.0

        def dH(t, sig):
            d = np.einsum("kii->ki", sig).real
            out = np.zeros(sig.shape, dtype=np.complex128)
            idx = np.arange(sig.shape[-1])
            out[:, idx, idx] = U * (d - 0.5)
            return out
        return dH

    def bias_source(self) -> str:
        """Source text of an equivalent ``Bias.py`` (reference callback names)."""
        b = self.bias
        lines = ["import numpy as np", "_SPEC = " + repr(dict(b))]
        lines.append("def bias(t, a):")
        lines.append("    " + _bias_expr(b))
        if self.hubbard_U is None:
            lines.append("def dH(t, sig):\n    return 0.0")
        else:
            lines.append("def dH(t, sig):")
            lines.append("    d = np.einsum('kii->ki', sig).real")
            lines.append("    out = np.zeros(sig.shape, dtype=np.complex128)")
            lines.append("    i = np.arange(sig.shape[-1])")
            lines.append("    out[:, i, i] = %r * (d - 0.5)" % float(self.hubbard_U))
            lines.append("    return out")
        lines.append("def dissipator(t, sig):\n    return 0.0")
        return "\n".join(lines) + "\n"


def _bias_expr(b: dict) -> str:
    k = b["kind"]
    if k == "exp_ramp":
        v = "%r*(1.0-np.exp(-t/%r))" % (b["V0"], b["tau"])
        return "V = %s\n    return V/2 if a == 0 else (-V/2 if a == 1 else 0.0)" % v
    if k == "gauss":
        v = "%r*np.exp(-(t-%r)**2/(2*%r**2))" % (b["V0"], b["tc"], b["sigma"])
        return "V = %s\n    return V/2 if a == 0 else (-V/2 if a == 1 else 0.0)" % v
    if k == "sin":
        v = "%r*np.sin(2*np.pi*%r*t)" % (b["V0"], b["f"])
        return "V = %s\n    return V/2 if a == 0 else (-V/2 if a == 1 else 0.0)" % v
    if k == "step_lead0":
        return "return %r if (a == 0 and t > 0.0) else 0.0" % b["V0"]
    if k == "zero":
        return "return 0.0"
    raise ValueError(k)


def bias_value(b: dict, t: float, a: int) -> float:
    """Lead bias Delta_a(t) in eV; the +/-V/2 split between leads 0 and 1 follows
    ``make_constant_bias`` (Zandpack/Pulses.py:81-88)."""
    k = b["kind"]
    if k == "step_lead0":
        return float(b["V0"]) if (a == 0 and t > 0.0) else 0.0
    if k == "zero":
        return 0.0
    if k == "exp_ramp":
        V = b["V0"] * (1.0 - math.exp(-t / b["tau"]))
    elif k == "gauss":
        V = b["V0"] * math.exp(-(t - b["tc"]) ** 2 / (2 * b["sigma"] ** 2))
    elif k == "sin":
        V = b["V0"] * math.sin(2 * math.pi * b["f"] * t)
    else:
        raise ValueError(k)
    if a == 0:
        return V / 2
    if a == 1:
        return -V / 2
    return 0.0


def _sort_pairs(e, v):
    order = np.argsort(-np.abs(e), kind="stable")
    e, v = e[order], v[:, order]
    if e.size:
        cut = 1e-12 * max(np.abs(e).max(), 1e-300)
        e = np.where(np.abs(e) < cut, 0.0, e)
    return e, v


def _sorted_eigh(M: np.ndarray):
    """Hermitian eigenpairs sorted by decreasing |eigenvalue|; eigenvalues below
    1e-12 of the largest are set to exactly zero."""
    e, v = np.linalg.eigh(M)
    return _sort_pairs(e, v)


def _sorted_eigh_stack(Ms: np.ndarray):
    """_sorted_eigh of every matrix of a stack, in one LAPACK loop (the same
    routine per matrix, so the same values as one call each)."""
    es, vs = np.linalg.eigh(Ms)
    return [_sort_pairs(es[i], vs[i]) for i in range(len(Ms))]


def build_arrays(H: np.ndarray, coupling: list, lor: list, n_pade: int, kT: float = 0.025,
                 mu: float = 0.0, zero_tol: float = 1e-10):
    """Assemble the ``Arrays`` dictionary.

    ``lor[a] = (centers, widths, G)`` with ``G`` of shape (N_L, n_c, n_c): the
    Lorentzian fit of lead ``a`` on its coupling orbitals ``coupling[a]``.
    """
    n = H.shape[0]
    L = len(coupling)
    N_L = len(lor[0][0])
    NF = n_pade
    NX = N_L + 2 * NF
    beta = 1.0 / kT
    z, eta = psd_poles(NF)
    nc_max = max(len(c) for c in coupling)
    # eigen axis before truncation: n_c of each lead
    GGP = np.zeros((1, L, NX, nc_max), complex)
    GGM = np.zeros_like(GGP); GLP = np.zeros_like(GGP); GLM = np.zeros_like(GGP)
    Xpp = np.zeros_like(GGP); Xpm = np.zeros_like(GGP)
    vec = np.zeros((L, NX, nc_max, nc_max), complex)   # eigenvectors on coupling orbitals
    for a in range(L):
        cen, wid, G = lor[a]
        nc = len(coupling[a])
        lor_pairs = _sorted_eigh_stack(G[:N_L]) if N_L else []
        for x in range(N_L):
            e, v = lor_pairs[x]
            epsx = np.array([cen[x] + 1j * wid[x]])
            fp = fermi_expanded(epsx, z, eta, beta, mu)[0]
            fm = fermi_expanded(epsx.conj(), z, eta, beta, mu)[0]
            W = wid[x]
            GGP[0, a, x, :nc] = -0.5j * e * W * (1 - fp)
            GGM[0, a, x, :nc] = -0.5j * e * W * (1 - fm)
            GLP[0, a, x, :nc] = 0.5j * e * W * fp
            GLM[0, a, x, :nc] = 0.5j * e * W * fm
            Xpp[0, a, x, :] = epsx[0]
            Xpm[0, a, x, :] = epsx[0].conj()
            vec[a, x, :nc, :nc] = v.T
        poles_p = mu + z * kT
        poles_m = mu - z * kT

        def gamma_at(zz):
            s = wid ** 2 / ((zz - cen) ** 2 + wid ** 2)
            return np.tensordot(s, G, axes=(0, 0))
        # Hermitian (part 0) and anti-Hermitian / i (part 1) parts of Gamma at the poles
        Ms_p, Ms_m = [], []
        for p in range(NF):
            for part in range(2):
                gp = gamma_at(poles_p[p])
                gm = gamma_at(poles_m[p])
                if part == 0:
                    Ms_p.append((gp + gp.conj().T) / 2)
                    Ms_m.append((gm + gm.conj().T) / 2)
                else:
                    Ms_p.append((gp - gp.conj().T) / 2j)
                    Ms_m.append((gm - gm.conj().T) / 2j)
        pairs_p = _sorted_eigh_stack(np.array(Ms_p)) if NF else []
        pairs_m = _sorted_eigh_stack(np.array(Ms_m)) if NF else []
        for p in range(NF):
            for part in range(2):  # 0: B (Hermitian part), 1: C (anti-Hermitian part / i)
                ep, vp = pairs_p[2 * p + part]
                em, _ = pairs_m[2 * p + part]
                if part == 1:
                    ep = 1j * ep
                    em = 1j * em
                x = N_L + part * NF + p
                GGP[0, a, x, :nc] = +eta[p] * ep / beta
                GLP[0, a, x, :nc] = +eta[p] * ep / beta
                GGM[0, a, x, :nc] = -eta[p] * em / beta
                GLM[0, a, x, :nc] = -eta[p] * em / beta
                Xpp[0, a, x, :] = poles_p[p]
                Xpm[0, a, x, :] = poles_m[p]
                vec[a, x, :nc, :nc] = vp.T
    # NOT: largest eigen index with a non-negligible entry, +1
    # (find_max_orbital_idx_per_lead, Zandpack/mpi_splitter.py:555-580)
    live = (np.abs(GGP[0]) >= zero_tol) | (np.abs(GLP[0]) >= zero_tol)
    NOT = int(max(np.where(live[a])[1].max() + 1 for a in range(L)))
    xi = np.zeros((1, L, NX, NOT, n), complex)
    for a in range(L):
        nc = len(coupling[a])
        cidx = np.asarray(coupling[a])
        for c in range(min(NOT, nc)):
            xi[0, a, :, c, cidx] = vec[a, :, c, :nc].T
    sl = (slice(None), slice(None), slice(None), slice(0, NOT))
    e, U = np.linalg.eigh(H)
    f = 1.0 / (1.0 + np.exp((e - mu) / kT))
    DM = (U * f) @ U.conj().T
    A = dict(
        H_Ortho=H[None].astype(np.complex128),
        DM_Ortho=DM[None].astype(np.complex128),
        psi_shape=np.array([1, L, NX, NOT, n]),
        Xpp=Xpp[sl].copy(), Xpm=Xpm[sl].copy(),
        GG_P=GGP[sl].copy(), GL_P=GLP[sl].copy(), GG_M=GGM[sl].copy(), GL_M=GLM[sl].copy(),
        diff_GGP_GLP=(GGP - GLP)[sl].copy(), diff_GGM_GLM=(GGM - GLM)[sl].copy(),
        xi=xi, Ixi=xi.conj(), zero_tol=np.array(zero_tol),
        num_leads=np.array(L), num_poles_fermi=np.array(NF), num_lorentzians=np.array(N_L),
        noT=np.array(NOT), kT_i=np.full(L, kT), mu_i=np.full(L, mu),
    )
    return A


def _lorentzians(rng, n_l, nc, rank, amp_lo=0.05, amp_hi=0.3, scale=None):
    cen = rng.uniform(-3, 3, n_l)
    wid = rng.uniform(0.1, 0.5, n_l)
    G = np.zeros((n_l, nc, nc), complex)
    for x in range(n_l):
        if nc == 1 and rank == 1:
            G[x, 0, 0] = rng.uniform(amp_lo, amp_hi)
            continue
        F = (rng.standard_normal((nc, rank)) + 1j * rng.standard_normal((nc, rank))) / math.sqrt(2)
        M = F @ F.conj().T
        target = scale if scale is not None else rng.uniform(amp_lo, amp_hi)
        M *= target / np.linalg.eigvalsh(M).max()
        G[x] = (M + M.conj().T) / 2
    return cen, wid, G


def _cfg_c1(rng):
    n = 20
    H = chain(n, -2.7)
    coupling = [[0], [n - 1]]
    lor = [_lorentzians(rng, 16, 1, 1) for _ in coupling]
    A = build_arrays(H, coupling, lor, 20)
    return A, coupling, dict(t0=0.0, t1=50.0, eps=1e-10, stepsize=0.01,
                             bias={"kind": "exp_ramp", "V0": 0.5, "tau": 5.0}, hubbard_U=None)


def _cfg_c2(rng):
    ncol, nrow = 16, 16
    H = honeycomb_ribbon(ncol, nrow, -2.7)
    H = H + np.diag(rng.uniform(-0.1, 0.1, ncol * nrow))
    coupling = [list(range(nrow)), list(range((ncol - 1) * nrow, ncol * nrow))]
    lor = [_lorentzians(rng, 32, nrow, 4, scale=0.1) for _ in coupling]
    A = build_arrays(H, coupling, lor, 40)
    return A, coupling, dict(t0=0.0, t1=40.0, eps=1e-7, stepsize=0.01,
                             bias={"kind": "gauss", "V0": 0.3, "tc": 20.0, "sigma": 5.0}, hubbard_U=None)


def _cfg_c3(rng):
    nx = ny = 32
    H = square_lattice(nx, ny, -1.0)
    coupling = [list(range(ny)), list(range((nx - 1) * ny, nx * ny))]
    lor = [_lorentzians(rng, 40, ny, 8) for _ in coupling]
    A = build_arrays(H, coupling, lor, 30)
    return A, coupling, dict(t0=0.0, t1=200.0, eps=1e-6, stepsize=0.01,
                             bias={"kind": "sin", "V0": 0.2, "f": 0.05}, hubbard_U=2.0)


def _cfg_c5(rng):
    n = 2048
    H = random_sparse(n, rng, 0.5, 2.7)
    coupling = [list(range(a * 512, a * 512 + 72)) for a in range(4)]
    lor = [_lorentzians(rng, 24, 72, 8) for _ in coupling]
    A = build_arrays(H, coupling, lor, 40)
    return A, coupling, dict(t0=0.0, t1=100.0, eps=1e-6, stepsize=0.01,
                             bias={"kind": "step_lead0", "V0": 0.4}, hubbard_U=None)


def _cfg_mini2(rng):
    """Small case with every feature of the n=1024 workload: 2D lattice, n_c=3,
    rank-2 Lorentzians, Hubbard dH(sigma), sinusoidal bias."""
    nx, ny = 4, 3
    H = square_lattice(nx, ny, -1.0)
    coupling = [list(range(ny)), list(range((nx - 1) * ny, nx * ny))]
    lor = [_lorentzians(rng, 4, ny, 2) for _ in coupling]
    A = build_arrays(H, coupling, lor, 3)
    return A, coupling, dict(t0=0.0, t1=2.0, eps=1e-8, stepsize=0.01,
                             bias={"kind": "sin", "V0": 0.4, "f": 0.2}, hubbard_U=2.0)


def _cfg_mini3(rng):
    """Three leads on a random sparse device, step bias on lead 0."""
    n = 14
    H = random_sparse(n, rng, 0.5, 2.7)
    coupling = [[0, 1], [5, 6, 7], [11, 12]]
    lor = [_lorentzians(rng, 3, len(c), 2) for c in coupling]
    A = build_arrays(H, coupling, lor, 2)
    return A, coupling, dict(t0=0.0, t1=1.0, eps=1e-8, stepsize=0.01,
                             bias={"kind": "step_lead0", "V0": 0.4}, hubbard_U=None)


CONFIGS = {
    "c1": (1, _cfg_c1),
    "c2": (2, _cfg_c2),
    "c3": (3, _cfg_c3),
    "c5": (5, _cfg_c5),
    "mini2": (102, _cfg_mini2),
    "mini3": (103, _cfg_mini3),
}


# ------------------------------------------------------------ ensemble (c4)
C4_SIZES = [(64, (8, 8)), (128, (16, 8)), (256, (16, 16)), (384, (24, 16)), (512, (32, 16))]


def c4_requests(count=512, rate=50.0, seed=1004, t_span="pulse"):
    """Requests of the serving ensemble: Poisson arrivals at ``rate`` per
    second, device sizes n in {64,128,256,384,512} as 1D chains (n_c = 1) or
    2D lattices (8x8, 16x8, 16x16, 24x16, 32x16, n_c = W), 2-3 leads, 16-32
    Lorentzians of rank min(4, n_c), 20-40 Pade poles, Gaussian pulses with
    amplitude U[0.1, 1] V and width U[2, 20] fs centred at one width.  Each is
    propagated over its pulse, to centre + 3 widths (``t_span="pulse"``), or
    over ``t_span`` fs when that is a number."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    out = []
    for i in range(count):
        n, shape = C4_SIZES[int(rng.integers(len(C4_SIZES)))]
        out.append(dict(id=i, arrival=float(arrivals[i]), n=n, shape=shape,
                        geom="1d" if rng.random() < 0.5 else "2d", leads=int(rng.integers(2, 4)),
                        n_l=int(rng.integers(16, 33)), n_f=int(rng.integers(20, 41)),
                        amp=float(rng.uniform(0.1, 1.0)), width=float(rng.uniform(2.0, 20.0)),
                        seed=int(rng.integers(2 ** 31)), t1=0.0))
        out[-1]["t1"] = 4.0 * out[-1]["width"] if t_span == "pulse" else float(t_span)
    return out


def c4_coupling(req):
    n = req["n"]
    if req["geom"] == "1d":
        c = [[0], [n - 1], [n // 2]]
    else:
        lx, ly = req["shape"]
        c = [list(range(ly)), list(range((lx - 1) * ly, lx * ly)),
             [i * ly + (ly - 1) for i in range(1, lx - 1)][:ly]]
    return c[:req["leads"]]


def c4_workload(req) -> Workload:
    rng = np.random.default_rng(req["seed"])
    n = req["n"]
    if req["geom"] == "1d":
        H = chain(n, -2.7)
    else:
        H = square_lattice(req["shape"][0], req["shape"][1], -1.0)
    coupling = c4_coupling(req)
    lor = [_lorentzians(rng, req["n_l"], len(c), min(4, len(c))) for c in coupling]
    A = build_arrays(H, coupling, lor, req["n_f"])
    bias = {"kind": "gauss", "V0": req["amp"], "tc": req["width"], "sigma": req["width"]}
    return Workload(name="c4-%d" % req["id"], arrays=A, t0=0.0, t1=req["t1"], eps=1e-6, stepsize=0.02,
                    hbar=HBAR, bias=bias, hubbard_U=None, kT=0.025, coupling=coupling)


def c4_mode_estimate(req):
    """(N, Ns, nc) of a request without building it: live modes are the
    Lorentzian ranks plus the Fermi-pole modes (rank n_c each)."""
    cs = [len(c) for c in c4_coupling(req)]
    Ns = sum(req["n_l"] * min(4, c) for c in cs)
    N = Ns + sum(2 * req["n_f"] * c for c in cs)
    return N, Ns, max(cs)


def make_workload(name: str) -> Workload:
    k, fn = CONFIGS[name]
    rng = np.random.default_rng(1000 + k)
    A, coupling, p = fn(rng)
    return Workload(name=name, arrays=A, t0=p["t0"], t1=p["t1"], eps=p["eps"], stepsize=p["stepsize"],
                    hbar=HBAR, bias=p["bias"], hubbard_U=p["hubbard_U"], kT=0.025, coupling=coupling)


# ------------------------------------------------- non-orthogonal basis
def make_nonorth_workload(name: str, s: float = 0.08, phases: bool = False) -> Workload:
    """A workload of ``name`` posed in a non-orthogonal basis, for the
    ``nozand`` path (Zandpack/mpi/nozand:259-320).

    The named workload's H, xi, Ixi are taken as the NON-orthogonal quantities
    H', xi', Ixi' (H' banded, xi' on the coupling orbitals), with the overlap
    S = 1 + s * (the bond pattern of H'), real symmetric positive definite.
    The ``Arrays`` hold them in the Loewdin-orthogonal basis as the reference
    stores them (``S^(-0.5)`` is the Loewdin factor, Zandpack/Writer.py:83,229):
    ``H_Ortho = S^-1/2 H' S^-1/2``, ``xi`` rows ``S^-1/2 xi'``, ``Ixi`` rows
    ``Ixi' S^-1/2``; ``nozand`` maps them back (``S^1/2`` on both sides,
    ``transform_vec_Tv/vT``).  ``DM_Ortho`` is kept: ``nozand`` starts from
    ``S^-1/2 DM_Ortho S^-1/2``.  ``phases=True`` gives the bonds of S
    seeded random phases (a complex Hermitian overlap, as at a k-point away
    from Gamma)."""
    w = make_workload(name)
    A = dict(w.arrays)
    Hp = np.asarray(A["H_Ortho"])[0]
    n = Hp.shape[0]
    bonds = ((np.abs(Hp) > 0) & ~np.eye(n, dtype=bool)).astype(np.float64)
    if phases:
        up = np.triu(bonds, 1) * np.exp(1j * np.random.default_rng(2024).uniform(0, 2 * np.pi, (n, n)))
        bonds = up + up.conj().T
    S = np.eye(n) + s * bonds
    e, V = np.linalg.eigh(S)
    if e.min() <= 0.1:
        raise ValueError("overlap not safely positive definite (min eigenvalue %.3g)" % e.min())
    Sm05 = (V * e ** -0.5) @ V.conj().T
    Sm05 = (Sm05 + Sm05.conj().T) / 2
    A["H_Ortho"] = (Sm05 @ Hp @ Sm05)[None].astype(np.complex128)
    A["xi"] = np.asarray(A["xi"]) @ Sm05.T
    A["Ixi"] = np.asarray(A["Ixi"]) @ Sm05
    A["S^(-0.5)"] = Sm05[None].astype(np.complex128)
    return dataclasses.replace(w, name=w.name + "-nonorth", arrays=A)


# ------------------------------------------------------------ k-points
def make_kpoint_workload(name: str, nk: int = 2, spread: float = 0.2) -> Workload:
    """A workload of ``name`` with ``nk`` k-points (the leading NK axis of
    every array, Zandpack/mpi/zand:113-124): k-point 0 is the named model, the
    others add seeded random on-site energies in [-spread, spread] eV to H and
    take their own isolated-device Fermi density matrix; the lead quantities
    (poles, coupling coefficients, xi) are shared by all k-points."""
    w = make_workload(name)
    A = dict(w.arrays)
    H0 = np.asarray(A["H_Ortho"])[0]
    n = H0.shape[0]
    rng = np.random.default_rng(4000 + nk)
    Hs, DMs = [H0], [np.asarray(A["DM_Ortho"])[0]]
    for _ in range(1, nk):
        H = H0 + np.diag(rng.uniform(-spread, spread, n))
        e, U = np.linalg.eigh(H)
        f = 1.0 / (1.0 + np.exp(e / w.kT))
        Hs.append(H)
        DMs.append((U * f) @ U.conj().T)
    A["H_Ortho"] = np.array(Hs, np.complex128)
    A["DM_Ortho"] = np.array(DMs, np.complex128)
    for k in ("Xpp", "Xpm", "GG_P", "GL_P", "GG_M", "GL_M", "diff_GGP_GLP", "diff_GGM_GLM", "xi", "Ixi"):
        A[k] = np.repeat(np.asarray(A[k]), nk, axis=0)
    ps = np.array(A["psi_shape"])
    ps[0] = nk
    A["psi_shape"] = ps
    return dataclasses.replace(w, name="%s-k%d" % (w.name, nk), arrays=A)
