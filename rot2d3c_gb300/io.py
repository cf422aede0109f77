"""The reference's input and output file formats.

* ``parameter.inp``: 25 values read positionally with list-directed READ,
  then two directory names (Rot2D3C.para.f90:134-163);
* ``status.inp``: the last output index ``stat`` and its ``time``
  (Rot2D3C.para.f90:125-130);
* binary fields ``ps|vz|ww|invlap_psi.NNN.XXX.out``: gfortran sequential
  unformatted files, one record of n*n REAL*8 framed by 4-byte record-length
  markers (Rot2D3C.para.f90:483-519; the Python reader of the reference,
  python_scripts/field_calc.py:13-18, skips the first marker);
* text diagnostics written with Fortran ``Ew.dEe`` and ``Fw.d`` edit
  descriptors: ``energy_bal.txt`` & co. in E23.14E3
  (pseudospec2D_Rot2D3C.f90:592-609), spectra and transfers in E24.15E3
  (:703-709, :819-834), ``time_spec.txt`` / ``time_field.txt`` as A4,F12.6 and
  A3,F12.6 (Rot2D3C.para.f90:451-456, :521-528).
"""
from __future__ import annotations

import os
import struct
from decimal import ROUND_HALF_EVEN, Decimal

import numpy as np

# field order of parameter.inp (Rot2D3C.para.f90:136-160)
PARAM_ORDER = [
    ("cfl", float), ("step", int), ("cstep", int), ("sstep", int), ("tstep", int),
    ("fp0", float), ("fz0", float), ("u0", float), ("v0", float), ("kdn", float), ("kup", float),
    ("nu", float), ("hnu", float), ("nn", int), ("mm", int), ("nuv", float), ("hnuv", float),
    ("nnv", int), ("mmv", int), ("omega", float), ("seed", int), ("iflow", int), ("prm1", float),
    ("prm2", float), ("dt_corr", float),
]


def _first_value(line: str) -> str:
    """The value a list-directed READ of one item takes from a record: the
    first token before a blank, comma or slash."""
    tok = line.strip().replace(",", " ").split()
    if not tok:
        raise ValueError("empty record where a value was expected")
    return tok[0].split("/")[0]


def _fortran_number(tok: str, kind):
    t = tok.lower().replace("d", "e")
    if kind is int:
        return int(t)
    return float(t)


def read_parameter_inp(path: str) -> dict:
    """Positional reader of parameter.inp; returns a dict with the 25 values
    plus ``idir`` and ``odir`` (the 100-character directory records)."""
    with open(path) as f:
        lines = f.read().splitlines()
    if len(lines) < len(PARAM_ORDER) + 2:
        raise ValueError(f"{path}: expected {len(PARAM_ORDER) + 2} records, found {len(lines)}")
    out = {}
    for i, (name, kind) in enumerate(PARAM_ORDER):
        try:
            out[name] = _fortran_number(_first_value(lines[i]), kind)
        except ValueError as e:
            raise ValueError(f"{path}: record {i + 1} ({name}): {e}") from None
    out["idir"] = lines[len(PARAM_ORDER)][:100].rstrip()
    out["odir"] = lines[len(PARAM_ORDER) + 1][:100].rstrip()
    return out


def read_status_inp(path: str):
    """(stat, time) from status.inp."""
    with open(path) as f:
        lines = f.read().splitlines()
    if len(lines) < 2:
        raise ValueError(f"{path}: expected 2 records")
    return _fortran_number(_first_value(lines[0]), int), _fortran_number(_first_value(lines[1]), float)


def write_status_inp(path: str, stat: int, time: float) -> None:
    with open(path, "w") as f:
        f.write(f"{stat}           % last output file\n{time!r}         % time of last output\n")


# ------------------------------------------------------------------ binary
def write_field(path: str, r: np.ndarray) -> None:
    """One sequential unformatted record of REAL*8 R(n,n) (x fastest)."""
    a = np.ascontiguousarray(r, dtype="<f8")
    nbytes = a.nbytes
    if nbytes > 0x7FFFFFFF:
        raise ValueError("record larger than 2 GiB needs gfortran subrecords (n <= 8192 supported)")
    mark = struct.pack("<i", nbytes)
    with open(path, "wb") as f:
        f.write(mark)
        f.write(a.tobytes())
        f.write(mark)


def read_field(path: str, n: int) -> np.ndarray:
    """Inverse of write_field; checks both record markers."""
    with open(path, "rb") as f:
        raw = f.read()
    want = 8 * n * n
    if len(raw) != want + 8:
        raise ValueError(f"{path}: {len(raw)} bytes, expected {want + 8}")
    head, = struct.unpack("<i", raw[:4])
    tail, = struct.unpack("<i", raw[-4:])
    if head != want or tail != want:
        raise ValueError(f"{path}: record markers {head}/{tail}, expected {want}")
    return np.frombuffer(raw[4:-4], dtype="<f8").reshape(n, n).copy()


# ------------------------------------------------------------------ text
def fortran_e(x: float, w: int, d: int, e: int = 3) -> str:
    """Fortran Ew.dEe edit descriptor (gfortran): 0.ddd...E+xxx, right-aligned
    in w characters; decimal rounding to nearest (ties to even) on the exact
    binary value."""
    x = float(x)
    if x != x:
        return "NaN".rjust(w)
    if x in (float("inf"), float("-inf")):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    sign = "-" if (x < 0 or (x == 0 and str(x).startswith("-"))) else ""
    if x == 0.0:
        body = "0." + "0" * d + "E+" + "0" * e
    else:
        dec = Decimal(abs(x))
        exp10 = dec.adjusted() + 1  # 0.1 <= m < 1
        m = (dec.scaleb(-exp10)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        if m >= 1:
            exp10 += 1
            m = (dec.scaleb(-exp10)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
        digits = format(m, "f")  # "0.ddd"
        es = "+" if exp10 >= 0 else "-"
        body = f"{digits}E{es}{abs(exp10):0{e}d}"
    s = sign + body
    if len(s) > w:
        return "*" * w
    return s.rjust(w)


def fortran_f(x: float, w: int, d: int) -> str:
    """Fortran Fw.d edit descriptor."""
    s = format(Decimal(float(x)).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN), "f")
    if s.startswith("0.") and len(s) > w:
        s = s[1:]
    if s.startswith("-0.") and len(s) > w:
        s = "-" + s[2:]
    return "*" * w if len(s) > w else s.rjust(w)


def e23_14(values) -> str:
    return "".join(fortran_e(v, 23, 14) for v in values)


def e24_15(values) -> str:
    return "".join(fortran_e(v, 24, 15) for v in values)


def append_cond_check(odir_cwd: str, out30) -> None:
    """Append the four balance lines of cond_check (pseudospec2D_Rot2D3C.f90:592-609)
    to energy_bal.txt, enstrophy_bal.txt, helicity_bal.txt and max_min.txt in
    the working directory ``odir_cwd``."""
    v = list(out30)
    for name, sl in (("energy_bal.txt", v[0:12]), ("enstrophy_bal.txt", v[12:17]),
                     ("helicity_bal.txt", v[17:25]), ("max_min.txt", v[25:30])):
        with open(os.path.join(odir_cwd, name), "a") as f:
            f.write(e23_14(sl) + "\n")


def write_spectrum(odir: str, ext4: str, ek, ezk) -> None:
    """spectrum.XXXX.txt: n/2+1 lines of Ek, Ezk (FORMAT 30, :699-709)."""
    with open(os.path.join(odir, f"spectrum.{ext4}.txt"), "w") as f:
        for a, b in zip(ek, ezk):
            f.write(e24_15((a, b)) + "\n")


def write_transfers(odir: str, ext4: str, fl0, fl1, fl2) -> None:
    """transfer.XXXX.txt (per shell) and fluxes.XXXX.txt (running sums)
    (FORMAT 40, :815-834)."""
    with open(os.path.join(odir, f"transfer.{ext4}.txt"), "w") as f:
        for a, b, c in zip(fl0, fl1, fl2):
            f.write(e24_15((a, b, c)) + "\n")
    fx0 = fx1 = fx2 = 0.0
    with open(os.path.join(odir, f"fluxes.{ext4}.txt"), "w") as f:
        for a, b, c in zip(fl0, fl1, fl2):
            fx0 = a + fx0
            fx1 = b + fx1
            fx2 = c + fx2
            f.write(e24_15((fx0, fx1, fx2)) + "\n")


def append_time_line(path: str, tag: str, time: float) -> None:
    """time_spec.txt (A4,F12.6) or time_field.txt (A3,F12.6)."""
    with open(path, "a") as f:
        f.write(tag + fortran_f(time, 12, 6) + "\n")


# ---------------------------------------------------------------------------
# Time averages of the outputs (python_scripts/SpectraAvg.py, FluxesAvg.py)
# ---------------------------------------------------------------------------
def _indexed(odir: str, head: str, start: int):
    """Files head.NNNN.txt of odir with NNNN >= start, in index order."""
    out = []
    for name in sorted(os.listdir(odir)):
        if name.startswith(head + ".") and name.endswith(".txt"):
            num = name[len(head) + 1:-4]
            if num.isdigit() and int(num) >= start:
                out.append(os.path.join(odir, name))
    return out


def _loadtxt(path: str) -> np.ndarray:
    return np.loadtxt(path, ndmin=2)


def mean_injection(run_dir: str, start: int, iflow: int):
    """Mean total energy and enstrophy injection from energy_bal.txt and
    enstrophy_bal.txt rows start.. (FluxesAvg.py:33-48): random forcing
    (iflow 3) halves the recorded injections."""
    e = _loadtxt(os.path.join(run_dir, "energy_bal.txt"))
    z = _loadtxt(os.path.join(run_dir, "enstrophy_bal.txt"))
    inj, injz, injenst = e[:, 3], e[:, 4], z[:, 2]
    if iflow == 3:
        inj, injz, injenst = inj / 2.0, injz / 2.0, injenst / 2.0
    return float(np.mean(inj[start:] + injz[start:])), float(np.mean(injenst[start:]))


def average_spectra(odir: str, start: int):
    """Mean (E_2D, E_z) over spectrum.NNNN.txt with NNNN >= start
    (SpectraAvg.py:35-60): each file weighted 1/number of files."""
    files = _indexed(odir, "spectrum", start)
    if not files:
        raise ValueError(f"no spectrum files with index >= {start} in {odir}")
    e2d = ez = None
    for f in files:
        d = _loadtxt(f)
        a, b = d[:, 0] / float(len(files)), d[:, 1] / float(len(files))
        e2d = a if e2d is None else e2d + a
        ez = b if ez is None else ez + b
    return e2d, ez


def average_fluxes(odir: str, start: int, injtot: float = 1.0, injenst: float = 1.0):
    """Mean (enstrophy flux / injenst, 2-D energy flux / injtot, vz energy
    flux / injtot) over fluxes.NNNN.txt with NNNN >= start (FluxesAvg.py:67-95)."""
    files = _indexed(odir, "fluxes", start)
    if not files:
        raise ValueError(f"no fluxes files with index >= {start} in {odir}")
    acc = None
    for f in files:
        d = _loadtxt(f)
        t = np.stack([d[:, 0] / injenst, d[:, 1] / injtot, d[:, 2] / injtot]) / float(len(files))
        acc = t if acc is None else acc + t
    return acc[0], acc[1], acc[2]
