"""The reference's file formats (CPU): positional parameter.inp/status.inp,
gfortran unformatted field records, Fortran E/F edit descriptors."""
import os
import struct

import numpy as np
import pytest

from rot2d3c_gb300 import io as fio

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_parameter_inp_positional():
    p = fio.read_parameter_inp(os.path.join(GOLD, "parameter_small.inp"))
    assert p["cfl"] == 0.3 and p["step"] == 7 and p["cstep"] == 2 and p["sstep"] == 3
    assert p["tstep"] == 4 and p["nu"] == 2e-3 and p["nuv"] == 1.5e-3 and p["nn"] == 1
    assert p["seed"] == 5 and p["iflow"] == 1 and p["omega"] == 0.5
    assert p["idir"] == "ins" and p["odir"] == "outs"
    assert fio.read_status_inp(os.path.join(GOLD, "status_small.inp")) == (0, 0.0)


def test_short_parameter_file_is_an_error(tmp_path):
    f = tmp_path / "parameter.inp"
    f.write_text("0.5\n10\n")
    with pytest.raises(ValueError):
        fio.read_parameter_inp(str(f))
    f.write_text("\n".join(["x"] * 27) + "\n")
    with pytest.raises(ValueError):
        fio.read_parameter_inp(str(f))


def test_field_record_round_trip(tmp_path):
    n = 16
    r = np.random.default_rng(0).standard_normal((n, n))
    path = str(tmp_path / "ps.000.001.out")
    fio.write_field(path, r)
    raw = open(path, "rb").read()
    assert len(raw) == 8 * n * n + 8
    assert struct.unpack("<i", raw[:4])[0] == 8 * n * n == struct.unpack("<i", raw[-4:])[0]
    # the reference's reader skips the 4-byte marker (field_calc.py:13-18)
    np.testing.assert_array_equal(np.frombuffer(raw[4:-4], "<f8").reshape(n, n), r)
    np.testing.assert_array_equal(fio.read_field(path, n), r)
    with open(path, "r+b") as f:
        f.write(struct.pack("<i", 12))
    with pytest.raises(ValueError):
        fio.read_field(path, n)


@pytest.mark.parametrize("x,w,d,s", [
    (1.0, 23, 14, "  0.10000000000000E+001"),
    (-0.123456789012345678, 23, 14, " -0.12345678901235E+000"),
    (0.0, 24, 15, "  0.000000000000000E+000"),
    (2.5e-5, 24, 15, "  0.250000000000000E-004"),
    (1e-300, 23, 14, "  0.10000000000000E-299"),
    (9.99999999999999999e5, 23, 14, "  0.10000000000000E+007"),
])
def test_fortran_e_descriptor(x, w, d, s):
    assert fio.fortran_e(x, w, d) == s
    assert float(s.replace("E", "e")) == pytest.approx(x, rel=10.0 ** -(d - 1), abs=1e-310)


def test_fortran_f_and_time_lines(tmp_path):
    assert fio.fortran_f(0.1234567, 12, 6) == "    0.123457"
    assert fio.fortran_f(-12.5, 12, 6) == "  -12.500000"
    p = str(tmp_path / "time_spec.txt")
    fio.append_time_line(p, "0001", 0.25)
    assert open(p).read() == "0001    0.250000\n"


def test_fluxes_are_running_sums(tmp_path):
    f0, f1, f2 = np.arange(5.0), -np.arange(5.0), np.ones(5)
    fio.write_transfers(str(tmp_path), "0001", f0, f1, f2)
    t = np.loadtxt(tmp_path / "transfer.0001.txt")
    x = np.loadtxt(tmp_path / "fluxes.0001.txt")
    np.testing.assert_allclose(t, np.c_[f0, f1, f2])
    np.testing.assert_allclose(x, np.c_[np.cumsum(f0), np.cumsum(f1), np.cumsum(f2)])
    assert len(open(tmp_path / "fluxes.0001.txt").readline()) == 3 * 24 + 1


def test_time_averages_of_spectra_and_fluxes(tmp_path):
    """average_spectra / average_fluxes / mean_injection (the reference's
    SpectraAvg.py, FluxesAvg.py) over files written by our own writers."""
    from rot2d3c_gb300 import io
    rng = np.random.default_rng(3)
    nb = 9
    spec, flx = [], []
    for i in range(1, 6):
        ek, ezk = rng.random(nb), rng.random(nb)
        f0, f1, f2 = rng.standard_normal(nb), rng.standard_normal(nb), rng.standard_normal(nb)
        ext = f"{i:04d}"
        io.write_spectrum(str(tmp_path), ext, ek, ezk)
        io.write_transfers(str(tmp_path), ext, f0, f1, f2)
        if i >= 3:
            spec.append((ek, ezk))
            flx.append((np.cumsum(f0), np.cumsum(f1), np.cumsum(f2)))
    e2d, ez = io.average_spectra(str(tmp_path), 3)
    np.testing.assert_allclose(e2d, np.mean([s[0] for s in spec], axis=0), rtol=1e-13)
    np.testing.assert_allclose(ez, np.mean([s[1] for s in spec], axis=0), rtol=1e-13)
    rows = np.column_stack([np.linspace(0, 1, 8)] + [rng.random(8) for _ in range(11)])
    np.savetxt(tmp_path / "energy_bal.txt", rows)
    zrows = np.column_stack([np.linspace(0, 1, 8)] + [rng.random(8) for _ in range(4)])
    np.savetxt(tmp_path / "enstrophy_bal.txt", zrows)
    inj, injz = io.mean_injection(str(tmp_path), 2, 3)
    assert inj == pytest.approx(np.mean(rows[2:, 3] + rows[2:, 4]) / 2)
    assert injz == pytest.approx(np.mean(zrows[2:, 2]) / 2)
    z, a, b = io.average_fluxes(str(tmp_path), 3, injtot=inj, injenst=injz)
    np.testing.assert_allclose(z, np.mean([f[0] for f in flx], axis=0) / injz, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(a, np.mean([f[1] for f in flx], axis=0) / inj, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(b, np.mean([f[2] for f in flx], axis=0) / inj, rtol=1e-12, atol=1e-14)
