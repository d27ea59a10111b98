"""DAC I/O and the spicule set-up against the reference's own output files.

The fixture tests/golden/spicule_reference.npz holds the arrays and SHA-256
digests of the DAC files, params.txt and out.txt that the reference ships
from one run of its spicule model (cans1d/md_spicule/hdmlw); it was made by
tests/golden/make_spicule_golden.py.  CPU only.
"""
import hashlib
import struct
from pathlib import Path

import numpy as np
import pytest

from utrip_gb300 import dac, drivers, setups

GOLD = Path(__file__).resolve().parent / "golden" / "spicule_reference.npz"
STATIC = ["x", "bx", "bxm", "sc", "scm", "gx", "gxm", "rr", "rrm"]
SERIES = ["ro", "pr", "vx", "vy", "by"]


@pytest.fixture(scope="module")
def ref():
    return dict(np.load(GOLD))


def _sha(path):
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


def test_writer_reproduces_every_reference_file_byte_for_byte(ref, tmp_path):
    for name in STATIC:
        rec = ref[f"{name}_records"]
        assert not ref[f"{name}_unlimited"] and rec.shape == (1, 1026)
        dac.write_1d(tmp_path / f"{name}.dac", rec[0])
        assert _sha(tmp_path / f"{name}.dac") == str(ref[f"{name}_sha256"]), name
    with dac.dacdef0s(tmp_path / "t.dac") as w:
        for v in ref["t_records"]:
            w.write(v)
    assert _sha(tmp_path / "t.dac") == str(ref["t_sha256"])
    for name in SERIES:
        with dac.dacdef1s(tmp_path / f"{name}.dac", 1026) as w:
            for r in ref[f"{name}_records"]:
                w.write(r)
        assert _sha(tmp_path / f"{name}.dac") == str(ref[f"{name}_sha256"]), name


def test_reader_round_trip_and_restart_record(ref, tmp_path):
    with dac.dacdef1s(tmp_path / "ro.dac", 1026) as w:
        for r in ref["ro_records"]:
            w.write(r)
    f = dac.dacopnr(tmp_path / "ro.dac", 1)
    assert f.mtype == dac.MTYPE_FLOAT64 and f.unlimited and f.dims == (1026,) and f.nx == 2
    assert np.array_equal(f.last().view(np.int64), ref["ro_records"][1].view(np.int64))
    with pytest.raises(dac.DacError):
        dac.dacopnr(tmp_path / "ro.dac", 2)  # the rank check of dacopnr2s


def test_reader_rejects_bad_headers(tmp_path):
    def rec(b):
        n = struct.pack("<i", len(b))
        return n + b + n

    def ints(*v):
        return rec(struct.pack("<%di" % len(v), *v))

    good = ints(1) + ints(0) + ints(6) + ints(2) + ints(3, -1) + rec(np.zeros(3).tobytes())
    (tmp_path / "ok.dac").write_bytes(good)
    assert dac.DacFile(tmp_path / "ok.dac").nx == 1
    cases = {
        "endian": ints(16777216) + good[12:],                       # byte-swapped probe
        "version": ints(1) + ints(1) + good[24:],
        "mtype": ints(1) + ints(0) + ints(7) + good[36:],
        "marker": good[:-4] + struct.pack("<i", 99),
        "short": good[:-10],
        "record": ints(1) + ints(0) + ints(6) + ints(2) + ints(3, -1) + rec(np.zeros(2).tobytes()),
    }
    for name, raw in cases.items():
        (tmp_path / f"{name}.dac").write_bytes(raw)
        with pytest.raises(dac.DacError):
            dac.DacFile(tmp_path / f"{name}.dac")
    with pytest.raises(dac.DacError):  # a fixed-size file holds one record
        with dac.dacdef1d(tmp_path / "d.dac", 3) as w:
            w.write(np.zeros(3))
            w.write(np.zeros(3))


def test_params_txt_byte_for_byte(ref, tmp_path):
    s = setups.spicule_1d()
    with dac.DacParams(tmp_path / "params.txt") as p:
        p.puti("ix", s["x"].size)
        p.puti("margin", s["margin"])
        p.putd("ztr", s["ztr"])
        p.putd("tcor", s["tcor"])
        p.putd("gm", s["gm"])
    assert (tmp_path / "params.txt").read_text() == str(ref["params_txt"])
    got = dac.read_params(tmp_path / "params.txt")
    assert got["ix"] == 1026 and got["margin"] == 1 and got["ztr"] == 15.0


def test_e20_13_and_e10_3_formats():
    assert dac._e20_13(5.0 / 3.0) == " 0.1666666666667E+01"
    assert dac._e20_13(-2.5e-7) == "-0.2500000000000E-06"
    assert dac._e20_13(0.0) == " 0.0000000000000E+00"
    assert drivers._e10_3(0.18685411175615266) == " 0.187E+00"
    assert drivers._e10_3(12.5) == " 0.125E+02"


def test_out_txt_lines(ref):
    t = ref["t_records"]
    lines = [drivers._out_line("write", 0, t[0], 1), drivers._out_line("write", 100000, t[1], 2),
             drivers._out_line("stop", 100000, t[1]), "   ### normal stop ###"]
    assert "\n".join(lines) + "\n" == str(ref["out_txt"])


def test_spicule_setup_matches_reference_initial_output(ref):
    """model.f + the set-up part of main.f against the t = 0 records.  The
    grid, the flux-tube radius and the velocities and field (including the
    -0.0 of the odd-symmetric vx ghost) agree bit for bit; the rest agrees to
    a few units in the 14th digit: the reference run evaluated each statement
    with 80-bit extended intermediates (see the next test), so its last bits
    are not those of a double-precision evaluation."""
    s = setups.spicule_1d()
    for name in ("x", "rr", "rrm"):
        assert np.array_equal(ref[f"{name}_records"][0].view(np.int64),
                              s[name].view(np.int64)), name
    for k, name in enumerate(s["names"]):
        r = ref[f"{name}_records"][0]
        if name in ("vx", "vy", "by"):
            assert np.array_equal(r.view(np.int64), s["state"][k].view(np.int64)), name
        else:
            assert np.max(np.abs(r - s["state"][k]) / np.abs(r)) < 5e-14, name
    for name in ("bx", "bxm", "sc", "scm", "gx", "gxm"):
        r = ref[f"{name}_records"][0]
        den = np.where(r == 0, 1.0, np.abs(r))
        assert np.max(np.abs(r - s[name]) / den) < 5e-16, name
    assert float(ref["t_records"][0]) == 0.0


@pytest.mark.skipif(np.finfo(np.longdouble).nmant != 63,
                    reason="needs the 80-bit x87 long double")
def test_reference_setup_used_extended_precision(ref):
    """The reference's bx(1) = sqrt(8 pi p) and its gravity profile are
    reproduced bit for bit when each statement is evaluated in 80-bit
    extended precision and rounded to double on assignment, and not in
    double precision: the evidence that the last-bit differences above come
    from the reference build's arithmetic, not from the set-up."""
    L = np.longdouble
    s = setups.spicule_1d()
    p = s["state"][1][1]  # p(1) = p(2): te = 1 at both cells
    pi = L(np.arccos(-1.0))
    bx_ext = float(np.sqrt(L(8) * pi * L(p)))
    assert bx_ext == float(ref["bx_records"][0][0])
    assert float(np.sqrt(8.0 * float(pi) * p)) != float(ref["bx_records"][0][0])
    x = s["x"]
    gl0 = L(1.0) / L(5.0 / 3.0)
    gx = np.array([float(-(L(float(gl0)) * (L(1.0) - np.tanh((L(v) - L(400.0)) / L(10.0)))) / 2)
                   for v in x])
    gx[0] = -gx[1]
    assert np.array_equal(gx.view(np.int64), ref["gx_records"][0].view(np.int64))
