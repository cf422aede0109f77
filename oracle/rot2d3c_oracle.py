"""CPU oracle for the Rot2D3C time-step hot path (FP64, NumPy).

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` use it, and only as the checker or
the timed CPU restatement.

Parity status: **parity unpinned**.  The reference (Fortran 90 + MPI + FFTW 2,
``src/makefile:10-20``) cannot be compiled in this environment (no Fortran
compiler, no MPI, no FFTW 2) and ships no tests, fixtures or golden vectors.
This module is a line-by-line restatement of the reference algorithm; each
function cites the reference file:line it follows.  It is anchored instead by
analytic known-answer tests (direct O(n^2) DFT sums for the FFT convention,
single-mode derivatives, the two-mode Poisson bracket, the linear decay factor,
the Coriolis 2x2 system) and by the randu integer recurrence.

Layout conventions (same as the reference, C-order views of Fortran arrays):

* spectral arrays: complex128 ``[kx][ky]`` with shape ``(n//2+1, n)``, ky
  fastest -- the Fortran ``C(n, n/2+1)`` of ``fftp2D.f90:153``;
* physical arrays: float64 ``[y][x]`` with shape ``(n, n)``, x fastest -- the
  Fortran ``R(n, n)`` of ``fftp2D.f90:157``.

The FFTs are unnormalised with forward sign -1 (``fftw_f77.i:7-11``); a
C2R(R2C(x)) round trip returns ``n**2 * x``.  FFTW 2 (unpinned version, not
vendored) computes the plain DFT; ``numpy.fft`` (pocketfft) computes the same
DFT, which is what the restatement relies on.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

# var module, pseudospec2D_mod.f90:34-39
PI = 3.1415926535897932384


# --------------------------------------------------------------------------
# randu: pseudospec2D_mod.f90:52-71
# --------------------------------------------------------------------------
_IQ, _IR, _MASK = 127773, 2836, 123459876
_IA, _IM = 16807, 2147483647
_AM = np.float32(1.0) / np.float32(_IM)  # REAL parameter am = 1./im (== 2**-31)


def _i32(x: int) -> int:
    x &= 0xFFFFFFFF
    return x - (1 << 32) if x & 0x80000000 else x


def randu(seed: list) -> float:
    """XOR-masked Park-Miller step (Schrage), pseudospec2D_mod.f90:63-69.

    ``seed`` is a one-element list standing for the Fortran INTEGER argument,
    which the routine updates in place.  The result is the REAL (float32)
    value in [-1, 1) returned as a Python float (promotion to DOUBLE as in the
    reference's mixed-mode expressions).
    """
    idum = _i32(seed[0] ^ _MASK)
    k = int(idum / _IQ)  # Fortran integer division truncates toward zero
    idum = _i32(_IA * (idum - k * _IQ) - _IR * k)
    if idum < 0:
        idum += _IM
    r = np.float32(_AM) * np.float32(idum)            # am*idum in REAL
    r = (np.float32(r) - np.float32(0.5)) * np.float32(2.0)
    seed[0] = _i32(idum ^ _MASK)
    return float(np.float32(r))


# --------------------------------------------------------------------------
# grid / wavenumbers: Rot2D3C.para.f90:213-228
# --------------------------------------------------------------------------
class Grid:
    """Wavenumber tables for an n x n grid (Rot2D3C.para.f90:213-228)."""

    def __init__(self, n: int):
        if n < 4 or n & (n - 1):
            raise ValueError("n must be a power of two >= 4")
        self.n = n
        self.kmax = (float(n) / 3.0) ** 2          # :213
        self.tiny = 0.000001                       # :214
        ka = np.empty(n)
        h = n // 2
        for i in range(1, h + 1):                  # :220-223
            ka[i - 1] = float(i - 1)
            ka[i + h - 1] = float(i - h - 1)
        self.ka = ka
        # ka2(j,i) = ka(i)**2 + ka(j)**2, i = kx column (0..n/2), j = ky row
        self.kx = ka[: h + 1]
        self.ka2 = self.kx[:, None] ** 2 + ka[None, :] ** 2   # :224-228
        # Hermitian weight of every half-plane sum: two=1 on the kx=0 column
        self.two = np.full((h + 1, 1), 2.0)
        self.two[0, 0] = 1.0
        self.nrm4 = float(n) ** 4

    @property
    def shape_spec(self):
        return (self.n // 2 + 1, self.n)

    @property
    def shape_phys(self):
        return (self.n, self.n)


# --------------------------------------------------------------------------
# FFTs: fftp2D.f90:133-290
# --------------------------------------------------------------------------
def r2c(g: Grid, r: np.ndarray) -> np.ndarray:
    """fftp2d_real_to_complex (fftp2D.f90:133-211): real x-FFT per y row
    (:171), transpose (:177-204), complex y-FFT per kx column (:208)."""
    c1 = np.fft.rfft(np.asarray(r, dtype=np.float64), axis=1)  # [y][kx]
    return np.ascontiguousarray(np.fft.fft(c1, axis=0).T)      # [kx][ky]


def c2r(g: Grid, c: np.ndarray) -> np.ndarray:
    """fftp2d_complex_to_real (fftp2D.f90:214-290): complex y-IFFT per kx
    column (:251), transpose (:255-282), real x-C2R per y row (:286).
    Unnormalised; the imaginary parts at kx=0 and kx=n/2 are ignored, as
    FFTW's complex-to-real transform does."""
    n = g.n
    t = np.fft.ifft(np.asarray(c, dtype=np.complex128), axis=1) * n  # [kx][y]
    t = np.ascontiguousarray(t.T)                                      # [y][kx]
    t[:, 0] = t[:, 0].real
    t[:, n // 2] = t[:, n // 2].real
    return np.fft.irfft(t, n=n, axis=1) * n


# --------------------------------------------------------------------------
# spectral elementwise operators: pseudospec2D_Rot2D3C.f90:6-127
# --------------------------------------------------------------------------
def derivk2(g: Grid, a: np.ndarray, dir: int) -> np.ndarray:
    """derivk2 (pseudospec2D_Rot2D3C.f90:6-68): i*kx*a (dir 1), i*ky*a
    (dir 2) or a copy (dir 0), zeroed where ka2 > kmax."""
    keep = g.ka2 <= g.kmax
    if dir == 1:
        k = np.broadcast_to(g.kx[:, None], a.shape)
    elif dir == 2:
        k = np.broadcast_to(g.ka[None, :], a.shape)
    else:
        return np.where(keep, a, 0.0 + 0.0j)
    # im*ka*a evaluated as (0,ka)*(ar,ai) = (-ka*ai, ka*ar)
    b = np.empty(a.shape, dtype=np.complex128)
    b.real = -k * a.imag
    b.imag = k * a.real
    return np.where(keep, b, 0.0 + 0.0j)


def laplak2(g: Grid, a: np.ndarray) -> np.ndarray:
    """laplak2 (:71-95): b = -ka2*a, no truncation."""
    m = -g.ka2
    b = np.empty(a.shape, dtype=np.complex128)
    b.real = m * a.real
    b.imag = m * a.imag
    return b


def inv_laplak2(g: Grid, a: np.ndarray) -> np.ndarray:
    """inv_laplak2 (:98-127): b = -a/ka2 where ka2 > tiny, else 0."""
    ok = g.ka2 > g.tiny
    d = np.where(ok, g.ka2, 1.0)
    b = np.empty(a.shape, dtype=np.complex128)
    b.real = -a.real / d
    b.imag = -a.imag / d
    return np.where(ok, b, 0.0 + 0.0j)


def poisson(g: Grid, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """poisson (:169-226): [a,b] = da/dx db/dy - da/dy db/dx in real space,
    divided by n**4 (:214) and transformed back (:217).  The trailing mask
    (:218-224) tests ka2>=kmax .and. ka2<=tiny, which never holds: no-op."""
    r1 = c2r(g, derivk2(g, a, 1))
    r2 = c2r(g, derivk2(g, b, 2))
    r3 = r1 * r2
    r1 = c2r(g, derivk2(g, a, 2))
    r2 = c2r(g, derivk2(g, b, 1))
    r3 = (r3 - r1 * r2) / g.nrm4
    return r2c(g, r3)


# --------------------------------------------------------------------------
# reductions: pseudospec2D_Rot2D3C.f90:336-451
# --------------------------------------------------------------------------
def _powi(x: np.ndarray, k: int) -> np.ndarray:
    """Fortran REAL**INTEGER (0**0 == 1; negative powers as 1/x**|k|)."""
    if k == 0:
        return np.ones_like(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        p = x ** abs(k)
        return 1.0 / p if k < 0 else p


def energy(g: Grid, a: np.ndarray, kin: int) -> float:
    """energy (:336-396): sum two*|a|^2*ka2**kin/n**4; kin>=0 sums every k
    (0**0 = 1), kin<0 only where ka2 >= tiny."""
    w = g.two * (np.abs(a) ** 2)
    if kin >= 0:
        return float(np.sum(w * _powi(g.ka2, kin) / g.nrm4))
    ok = g.ka2 >= g.tiny
    return float(np.sum(np.where(ok, w * _powi(np.where(ok, g.ka2, 1.0), kin), 0.0) / g.nrm4))


def inerprod(g: Grid, a: np.ndarray, b: np.ndarray, kin: int) -> float:
    """inerprod (:400-451): sum two*ka2**kin*Re(b*conj(a))/n**4 over
    ka2 <= kmax (kin>=0) or tiny <= ka2 <= kmax (kin<0)."""
    re = (b * np.conj(a)).real
    if kin >= 0:
        ok = g.ka2 <= g.kmax
        v = g.two * _powi(g.ka2, kin) * re
    else:
        ok = (g.ka2 <= g.kmax) & (g.ka2 >= g.tiny)
        v = g.two * _powi(np.where(ok, g.ka2, 1.0), kin) * re
    return float(np.sum(np.where(ok, v, 0.0) / g.nrm4))


def shell_index(g: Grid) -> np.ndarray:
    """kmn = int(sqrt(ka2)+.5) (:652)."""
    return (np.sqrt(g.ka2) + 0.5).astype(np.int64)


def spectrum(g: Grid, ps: np.ndarray, vz: np.ndarray):
    """spectrum (:615-712): shell sums Ek(kmn) += two*ka2*|ps|^2/n^4 and
    Ezk(kmn) += two*|vz|^2/n^4 for kmn in 1..n/2+1.  Returns (Ek, Ezk) with
    Ek[i-1] the Fortran Ek(i)."""
    nb = g.n // 2 + 1
    kmn = shell_index(g)
    ok = (kmn > 0) & (kmn <= nb)
    e = np.where(ok, g.two * g.ka2 * np.abs(ps) ** 2 / g.nrm4, 0.0)
    ez = np.where(ok, g.two * np.abs(vz) ** 2 / g.nrm4, 0.0)
    idx = np.where(ok, kmn - 1, 0)
    ek = np.bincount(idx.ravel(), weights=e.ravel(), minlength=nb)[:nb]
    ezk = np.bincount(idx.ravel(), weights=ez.ravel(), minlength=nb)[:nb]
    return ek, ezk


def transfers(g: Grid, ps: np.ndarray, vz: np.ndarray):
    """transfers (:715-837): c2 = [ps, -k^2 ps], c1 = [ps, vz];
    Fl0 += two*ka2*Re(ps conj c2)/n^4, Fl1 += two*Re(ps conj c2)/n^4,
    Fl2 -= two*Re(vz conj c1)/n^4, per shell.  Returns (Fl0, Fl1, Fl2)."""
    nb = g.n // 2 + 1
    c1 = laplak2(g, ps)
    c2 = poisson(g, ps, c1)
    c1 = poisson(g, ps, vz)
    kmn = shell_index(g)
    ok = (kmn > 0) & (kmn <= nb)
    idx = np.where(ok, kmn - 1, 0).ravel()
    f0 = np.where(ok, g.two * g.ka2 * (ps * np.conj(c2)).real / g.nrm4, 0.0)
    f1 = np.where(ok, g.two * (ps * np.conj(c2)).real / g.nrm4, 0.0)
    f2 = np.where(ok, -g.two * (vz * np.conj(c1)).real / g.nrm4, 0.0)
    out = [np.bincount(idx, weights=f.ravel(), minlength=nb)[:nb] for f in (f0, f1, f2)]
    return tuple(out)


def fluxes(fl0, fl1, fl2):
    """Cumulative sums written to fluxes.XXXX.txt (:824-830)."""
    return np.cumsum(fl0), np.cumsum(fl1), np.cumsum(fl2)


@dataclass
class Params:
    """The 25 positional values of parameter.inp (Rot2D3C.para.f90:136-160)
    plus the grid size n (module grid, pseudospec2D_mod.f90:7-14)."""
    n: int = 64
    cfl: float = 0.5
    step: int = 1
    cstep: int = 100
    sstep: int = 1000
    tstep: int = 10000
    fp0: float = 1.0
    fz0: float = 1.0
    u0: float = 0.01
    v0: float = 0.01
    kdn: float = 12.0
    kup: float = 12.0
    nu: float = 0.001
    hnu: float = 1.0
    nn: int = 1
    mm: int = 2
    nuv: float = 0.001
    hnuv: float = 1.0
    nnv: int = 1
    mmv: int = 2
    omega: float = 0.0
    seed: int = 1
    iflow: int = 3
    prm1: float = 1.0
    prm2: float = 1.0
    dt_corr: float = 0.0
    idir: str = "../ins"
    odir: str = "../outs"


def cond_check(g: Grid, p: Params, ps, vz, fp, fz, time: float) -> np.ndarray:
    """cond_check (:455-612).  Returns the 30 values written per call, in file
    order: energy_bal (12), enstrophy_bal (5), helicity_bal (8), max_min (5)
    (:594, :598, :602, :606)."""
    Ep1 = energy(g, ps, 1)
    injp1 = inerprod(g, ps, fp, 1)
    Dsp = energy(g, ps, p.nn + 1)
    Hds = energy(g, ps, 1 - p.mm)
    Epv = energy(g, vz, 0)
    injz = inerprod(g, vz, fz, 0)
    Dspv = energy(g, vz, p.nnv)
    Hdsv = energy(g, vz, -p.mmv)
    C1 = derivk2(g, ps, 2)
    coup = inerprod(g, vz, C1, 0)
    Ep2 = energy(g, ps, 2)
    injp2 = inerprod(g, ps, fp, 2)
    Dspw = energy(g, ps, p.nn + 2)
    Hdsw = energy(g, ps, 2 - p.mm)
    Eph = inerprod(g, vz, ps, 1)
    injh1 = inerprod(g, vz, fp, 1)
    injh2 = inerprod(g, ps, fz, 1)
    Dsph1 = inerprod(g, vz, ps, p.nn + 1)
    Hdsh1 = inerprod(g, vz, ps, 1 - p.mm)
    Dsph2 = inerprod(g, ps, vz, p.nnv + 1)
    Hdsh2 = inerprod(g, ps, vz, 1 - p.mmv)
    # energy in the kup band (:551-568)
    kk = p.kup * p.kup
    band = (g.ka2 <= 2.01 * kk) & (g.ka2 >= kk)
    Efp = float(np.sum(np.where(band, g.two * g.ka2 * np.abs(ps) ** 2 / g.nrm4, 0.0)))
    Efpz = float(np.sum(np.where(band, g.two * np.abs(vz) ** 2 / g.nrm4, 0.0)))
    # extrema of -W and vz in real space (:573-586)
    R1 = c2r(g, laplak2(g, ps))
    maxw, minw = float(R1.max()), float(R1.min())
    R1 = c2r(g, derivk2(g, vz, 0))
    maxv, minv = float(R1.max()), float(R1.min())
    w = 2 * p.omega
    return np.array([
        time, Ep1, Epv, injp1, injz, p.nu * Dsp, p.nuv * Dspv, p.hnu * Hds,
        p.hnuv * Hdsv, w * coup, Efp, Efpz,
        time, Ep2, injp2, p.nu * Dspw, p.hnu * Hdsw,
        time, -Eph, -injh1, -injh2, -p.nu * Dsph1, -p.nuv * Dsph2,
        -p.hnu * Hdsh1, -p.hnuv * Hdsh2,
        time, maxw, minw, maxv, minv,
    ])


def cfl_condition(g: Grid, p: Params, ps, vz) -> float:
    """CFL_condition (:840-899).  The max of vz^2 (:879-888) is computed by
    the reference but not used in dt (:895), so it is not computed here."""
    n = g.n
    kcut = float(n) / 3.0
    nrm = float(n) ** 2
    r1 = c2r(g, derivk2(g, ps, 1))
    r2 = c2r(g, derivk2(g, ps, 2))
    tmp1 = float(np.max(r1 * r1 + r2 * r2))
    tmp = math.sqrt(tmp1) / nrm
    return p.cfl / (kcut * tmp + p.nu * (kcut ** (2 * p.nn))
                    + p.nuv * (kcut ** (2 * p.nnv)) + 2 * p.omega)


# --------------------------------------------------------------------------
# forcing: Rot2D3C.para.f90:343-381, pseudospec2D_Rot2D3C.f90:977-1126
# --------------------------------------------------------------------------
def rand_force(g: Grid, kdn: float, kup: float, fp0: float, dt: float,
               seed: list, kin: int) -> np.ndarray:
    """rand_force (:1063-1126), one rank.  ``seed`` advances by one randu
    call: the second draw uses the temporary ``seed+1`` (:1088)."""
    n = g.n
    theta = randu(seed) * PI
    phase = randu([seed[0] + 1]) * PI
    kx = float(math.floor(kup * math.cos(theta) + 0.5))
    ky = float(math.floor(kup * math.sin(theta) + 0.5))
    tmp = math.sqrt(2.0 * fp0) / (math.sqrt(dt) * kup ** kin)
    tmp1 = tmp * math.cos(phase)
    tmp2 = tmp * math.sin(phase)
    val = complex(tmp1, tmp2) * float(n) ** 2
    fp = np.zeros(g.shape_spec, dtype=np.complex128)
    ka = g.ka
    for i in range(1, n // 2 + 1):          # Fortran columns i = 2..n/2+1
        kai = g.kx[i]
        if kai == ky or kai == -ky:
            for j in range(n):
                if ka[j] == kx:
                    fp[i, j] = val
    if g.kx[0] == ky:                         # column i = 1 (:1109-1121)
        for j in range(1, n // 2):
            if ka[j] == kx:
                fp[0, j] = val
                fp[0, n - j] = np.conj(val)
    return fp


def const_inj(g: Grid, ps, kdn: float, kup: float, fp0: float, kin: int,
              seed: list, myrank: int = 0) -> np.ndarray:
    """const_inj (:977-1060), one rank.  Builds fp = ps/(|ps|^2+1) in the
    band kdn^2 <= ka2 <= kup^2 (Hermitian fill on kx=0), takes
    Efp = inerprod(ps, fp, kin), then fp = fp*fp0/Efp + i*randu*|k|*ps with
    randu seeded from myrank (the caller's seed is overwritten, :1032)."""
    n = g.n
    lo, hi = kdn * kdn, kup * kup
    fp = np.zeros(g.shape_spec, dtype=np.complex128)
    band = (g.ka2 <= hi) & (g.ka2 >= lo)
    base = ps / (np.abs(ps) ** 2 + 1.0)
    fp[1:] = np.where(band[1:], base[1:], 0.0)
    for j in range(1, n // 2):
        if band[0, j]:
            fp[0, j] = base[0, j]
            fp[0, n - j] = np.conj(base[0, j])
        else:
            fp[0, j] = 0.0
            fp[0, n - j] = 0.0
    fp[0, 0] = 0.0
    fp[0, n // 2] = 0.0
    Efp = inerprod(g, ps, fp, kin)
    seed[0] = myrank
    out = np.zeros_like(fp)
    for i in range(0, n // 2 + 1):
        if i != 0:
            for j in range(n):
                if band[i, j]:
                    t3 = randu(seed) * math.sqrt(g.ka2[i, j])
                    out[i, j] = fp[i, j] * fp0 / Efp + 1j * t3 * ps[i, j]
        else:
            for j in range(1, n // 2):
                if band[0, j]:
                    t3 = randu(seed) * math.sqrt(g.ka2[0, j])
                    out[0, j] = fp[0, j] * fp0 / Efp + 1j * t3 * ps[0, j]
                    out[0, n - j] = np.conj(out[0, j])
    return out


def forcing_iflow1(g: Grid, p: Params):
    """Deterministic forcing, iflow=1 (Rot2D3C.para.f90:343-371)."""
    n = g.n
    x = (np.arange(1, n + 1, dtype=np.float64) - 1.0)
    ax = 2 * p.kup * PI * x / float(n)
    R1 = np.sin(ax)[None, :] + np.sin(ax)[:, None]
    R2 = np.cos(ax)[None, :] + np.sin(ax)[:, None]
    fp = r2c(g, R1)
    eneru = energy(g, fp, 1)
    tmp = p.fp0 / math.sqrt(eneru)
    fz = r2c(g, R2)
    enerv = energy(g, fz, 0)
    tmp1 = p.fz0 / math.sqrt(enerv)
    m = (g.ka2 <= g.kmax) & (g.ka2 >= g.tiny)
    return np.where(m, tmp * fp, 0.0), np.where(m, tmp1 * fz, 0.0)


def initial_conditions(g: Grid, p: Params, seed: list):
    """Seeded initial condition for stat == 0 (Rot2D3C.para.f90:245-299).
    The loop bound kup+1 is a DOUBLE converted to INTEGER (truncation); kr
    uses the 1-based ir, jr as the reference does."""
    n = g.n
    R1 = np.zeros((n, n))
    R2 = np.zeros((n, n))
    xi = np.arange(1, n + 1, dtype=np.float64) - 1.0
    kmaxi = int(p.kup + 1)
    for ir in range(1, kmaxi + 1):
        for jr in range(1, kmaxi + 1):
            kr = math.sqrt(float(ir * ir + jr * jr))
            ph1 = randu(seed) * 2.0 * PI
            ph2 = randu(seed) * 2.0 * PI
            ph3 = randu(seed) * 2.0 * PI
            ph4 = randu(seed) * 2.0 * PI
            ax = 2.0 * (ir - 1) * PI * xi / float(n)
            ay = 2.0 * (jr - 1) * PI * xi / float(n)
            R1 += np.cos(ax + ph1)[None, :] * np.cos(ay + ph2)[:, None] / kr
            R2 += np.sin(ax + ph3)[None, :] * np.cos(ay + ph4)[:, None]
    ps = r2c(g, R1)
    vz = r2c(g, R2)
    ener = energy(g, ps, 1)
    enerv = energy(g, vz, 0)
    tmp = p.u0 / math.sqrt(ener)
    tmp1 = p.v0 / math.sqrt(enerv)
    m = (g.ka2 <= g.kmax) & (g.ka2 >= g.tiny)
    return np.where(m, tmp * ps, 0.0), np.where(m, tmp1 * vz, 0.0)


# --------------------------------------------------------------------------
# RK step: Rot2D3C.para.f90:545-611
# --------------------------------------------------------------------------
@dataclass
class Seeds:
    seed: list = field(default_factory=lambda: [1])
    seed1: list = field(default_factory=lambda: [2])


def rk_step(g: Grid, p: Params, ps, vz, fp, fz, dt: float, seeds: Seeds | None = None,
            ord: int = 4, tau5=None, tau6=None):
    """One low-storage RK step of order ``ord`` (Rot2D3C.para.f90:545-611)
    with semi-implicit divisor dissipation.  Returns the new (ps, vz) and,
    for iflow=2, the last forcing (fp, fz).  ``tau5``/``tau6`` (spectral,
    optional) are learned subgrid tendencies added to the two brackets (no
    counterpart in the reference)."""
    C1 = ps.copy()
    C2 = vz.copy()
    m = (g.ka2 <= g.kmax) & (g.ka2 > g.tiny)
    ka2 = g.ka2
    for o in range(ord, 0, -1):
        if p.iflow == 2:                                   # :565-569
            seeds.seed1[0] = seeds.seed[0] + 1
            fp = const_inj(g, C1, p.kdn, p.kup, p.fp0, 1, seeds.seed1)
            fz = const_inj(g, C2, p.kdn, p.kup, p.fz0, 0, seeds.seed)
        C4 = laplak2(g, C1)                                # :571
        C5 = poisson(g, C1, C4)                            # :572
        C6 = poisson(g, C1, C2)                            # :573
        if tau5 is not None:
            C5 = C5 + tau5
            C6 = C6 + tau6
        C3 = derivk2(g, C1, 2)                             # :575
        C4 = derivk2(g, C2, 2)                             # :576
        tmp1 = dt / float(o)                               # :581
        with np.errstate(divide="ignore", invalid="ignore"):
            tmp2 = np.where(m, 1.0 / np.where(m, ka2, 1.0), 0.0)   # :582
            tmp3 = 1.0 + (p.nu * _powi(ka2, p.nn) + p.hnu * _powi(tmp2, p.mm)) * tmp1
            u1 = ps + ((-C5 + (2 * p.omega) * C4) * tmp2 + fp) * tmp1
            n1 = (u1.real / tmp3) + 1j * (u1.imag / tmp3)
            tmp3v = 1.0 + (p.nuv * _powi(ka2, p.nnv) + p.hnuv * _powi(tmp2, p.mmv)) * tmp1
            u2 = vz + (C6 + (2 * p.omega) * C3 + fz) * tmp1
            n2 = (u2.real / tmp3v) + 1j * (u2.imag / tmp3v)
        C1 = np.where(m, n1, 0.0 + 0.0j)
        C2 = np.where(m, n2, 0.0 + 0.0j)
    return derivk2(g, C1, 0), derivk2(g, C2, 0), fp, fz    # :610-611


# --------------------------------------------------------------------------
# synthetic seeded inputs (no reference counterpart: the workloads' inputs)
# --------------------------------------------------------------------------
def random_phase_field(g: Grid, kmin: float, kmax_shell: float, slope: float,
                       rng: np.random.Generator) -> np.ndarray:
    """Hermitian random-phase spectral field with |a(k)| ~ k**slope in the
    shell kmin <= |k| <= kmax_shell, zero elsewhere, built as the R2C of a
    real field so the kx=0 column is exactly Hermitian."""
    n = g.n
    k = np.sqrt(g.ka2)
    shell = (k >= kmin) & (k <= kmax_shell)
    amp = np.where(shell, np.where(k > 0, k, 1.0) ** slope, 0.0)
    ph = rng.uniform(0.0, 2 * np.pi, size=g.shape_spec)
    c = amp * np.exp(1j * ph)
    r = c2r(g, c)
    a = r2c(g, r) / float(n) ** 2
    return np.where(shell, a, 0.0)


# --------------------------------------------------------------------------
# learned-closure data (no counterpart in the reference)
# --------------------------------------------------------------------------
def coarsen(gf: Grid, gc: Grid, a: np.ndarray) -> np.ndarray:
    """Sharp spectral filter of a fine spectral field onto the coarse grid:
    modes with kx^2 + ky^2 <= (nc/3)^2 kept, rescaled by (nc/nf)^2 (both
    grids carry the unnormalised R2C scaling)."""
    nf, nc = gf.n, gc.n
    out = np.zeros(gc.shape_spec, dtype=np.complex128)
    for i in range(nc // 2):
        for j in range(nc):
            ky = int(gc.ka[j])
            if i * i + ky * ky <= gc.kmax:
                out[i, j] = a[i, ky if ky >= 0 else nf + ky] * (nc / nf) ** 2
    return out


def closure_inputs(g: Grid, ps, vz) -> np.ndarray:
    """[n, n, 8]: omega = k^2 psi, vz, d/dx and d/dy of psi, omega, vz in
    physical units (C2R / n^2)."""
    n2 = float(g.n) ** 2
    om = -laplak2(g, ps)
    fields = [om, derivk2(g, vz, 0), derivk2(g, ps, 1), derivk2(g, ps, 2), derivk2(g, om, 1),
              derivk2(g, om, 2), derivk2(g, vz, 1), derivk2(g, vz, 2)]
    return np.stack([c2r(g, f) / n2 for f in fields], axis=-1)


def closure_targets(gf: Grid, gc: Grid, psf, vzf) -> np.ndarray:
    """[nc, nc, 2]: P_c([psi,-k^2 psi]_f) - [psi_c,-k^2 psi_c] and
    P_c([psi,vz]_f) - [psi_c,vz_c], physical units."""
    psc, vzc = coarsen(gf, gc, psf), coarsen(gf, gc, vzf)
    t5 = coarsen(gf, gc, poisson(gf, psf, laplak2(gf, psf))) - poisson(gc, psc, laplak2(gc, psc))
    t6 = coarsen(gf, gc, poisson(gf, psf, vzf)) - poisson(gc, psc, vzc)
    n2 = float(gc.n) ** 2
    return np.stack([c2r(gc, t5) / n2, c2r(gc, t6) / n2], axis=-1)


# ---------------------------------------------------------------------------
# regrid_slices.f90 (a stand-alone program of the reference)
# ---------------------------------------------------------------------------
def regrid_slices(vold: np.ndarray, n: int, m: int, nnodes: int, mnodes: int) -> np.ndarray:
    """The reference's slice loops restated literally (regrid_slices.f90:62-115):
    the n x n field is split into nnodes slices of ns = n/nnodes columns
    (Fortran Vold(n, ns), x fastest), each old slice gives mnodes/nnodes new
    slices of ms = m/mnodes columns, Vnew(j, k) = Vold((j+1)*n/m,
    (k+(is-1)*ms+1)*n/m) with 1-based indices and integer division.  Input and
    output are row-major [y][x] (= Fortran R(x, y)); the new slices are
    concatenated in file order."""
    ns, ms = n // nnodes, m // mnodes
    out = np.empty((m, m))
    for inode in range(nnodes):
        vold_s = vold[inode * ns:(inode + 1) * ns, :]  # [k][j] = Vold(j, k)
        for is_ in range(1, mnodes // nnodes + 1):
            vnew = np.empty((ms, m))
            for k in range(1, ms + 1):
                k2 = (k + (is_ - 1) * ms + 1) * n // m
                for j in range(1, m + 1):
                    j2 = (j + 1) * n // m
                    vnew[k - 1, j - 1] = vold_s[k2 - 1, j2 - 1]
            slot = inode * (mnodes // nnodes) + is_ - 1
            out[slot * ms:(slot + 1) * ms, :] = vnew
    return out
