"""DAC files: the output and restart format of the CANS model packages.

Host-side mirror of the reference I/O library ``cansio``:

  dacdef0s / dacdef1s / dacdef2s / dacdef3s / dacdef4s   cansio/dacdef{0,1,2,3,4}s.f
  dacdef1d / dacdef2d / dacdef3d                        cansio/dacdef{1,2,3}d.f
  dacopnr0s / dacopnr1s / ... / dacopnr1d               cansio/dacopnr*.f
  dacdefparam, dacputparam{i,d,r,c}                     cansio/dacdefparam.f, dacputparam*.f
  dacgetparam{i,d,r,c}                                  cansio/dacgetparam*.f

A DAC data file is a Fortran unformatted sequential file (each record framed
by 4-byte little-endian length markers) holding five header records -- the
integer 1 (byte-order probe), 0 (format version), mtype (4 = int32,
5 = float32, 6 = float64, the IDL type code plus one), the rank and the
extents (-1 for the unlimited time axis of the ``*s`` kinds) -- followed by one
record per output step (``*s``) or a single record (``*d``).  The parameter
file ``params.txt`` holds formatted lines ``'#dac ',i4,a32,' ',value`` with
type 4 (i20), 5 (e20.13) or 2 (a20).

Arrays are written in Fortran order (first index fastest), which for the
state arrays of this package (x fastest) is the C order of an array indexed
[..., j, i].
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

MTYPE_INT32 = 4
MTYPE_FLOAT32 = 5
MTYPE_FLOAT64 = 6
_DTYPE = {MTYPE_INT32: np.dtype("<i4"), MTYPE_FLOAT32: np.dtype("<f4"),
          MTYPE_FLOAT64: np.dtype("<f8")}


class DacError(RuntimeError):
    """A DAC file that does not follow the format (the checks of dacopnr*.f)."""


def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


def _ints(*v: int) -> bytes:
    return _record(struct.pack("<%di" % len(v), *v))


class DacWriter:
    """An open DAC data file: the header is written on creation, each
    ``write`` appends one record (``write(idf) array`` in the reference)."""

    def __init__(self, path, mtype: int, dims, unlimited: bool):
        if mtype not in _DTYPE:
            raise DacError(f"mtype {mtype} is not 4, 5 or 6")
        self.path = Path(path)
        self.mtype = mtype
        self.dims = tuple(int(d) for d in dims)
        self.unlimited = unlimited
        self.count = int(np.prod(self.dims)) if self.dims else 1
        self._f = open(self.path, "wb")
        rank = len(self.dims) + (1 if unlimited else 0)
        ext = list(self.dims) + ([-1] if unlimited else [])
        # dacdef*.f: write(idf) 1 / 0 / mtype / rank / extents
        self._f.write(_ints(1) + _ints(0) + _ints(mtype) + _ints(rank) + _ints(*ext))
        self.records = 0

    def write(self, a) -> None:
        arr = np.asarray(a, dtype=_DTYPE[self.mtype])
        if arr.size != self.count:
            raise DacError(f"{self.path.name}: record of {arr.size} values, header says {self.count}")
        if not self.unlimited and self.records:
            raise DacError(f"{self.path.name}: a fixed-size file holds one record")
        # array in Fortran storage order: the first (x) index varies fastest
        self._f.write(_record(np.ascontiguousarray(arr).tobytes(order="C")))
        self.records += 1

    def flush(self) -> None:
        self._f.flush()

    def close(self) -> None:
        if not self._f.closed:
            self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def dacdef0s(path, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    """cansio/dacdef0s.f: a time series of scalars."""
    return DacWriter(path, mtype, (), True)


def dacdef1s(path, ix: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    """cansio/dacdef1s.f: a time series of ix values."""
    return DacWriter(path, mtype, (ix,), True)


def dacdef2s(path, ix: int, jx: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    return DacWriter(path, mtype, (ix, jx), True)


def dacdef3s(path, ix: int, jx: int, kx: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    return DacWriter(path, mtype, (ix, jx, kx), True)


def dacdef4s(path, ix: int, jx: int, kx: int, lx: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    return DacWriter(path, mtype, (ix, jx, kx, lx), True)


def dacdef1d(path, ix: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    """cansio/dacdef1d.f: one record of ix values (coordinates, static fields)."""
    return DacWriter(path, mtype, (ix,), False)


def dacdef2d(path, ix: int, jx: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    return DacWriter(path, mtype, (ix, jx), False)


def dacdef3d(path, ix: int, jx: int, kx: int, mtype: int = MTYPE_FLOAT64) -> DacWriter:
    return DacWriter(path, mtype, (ix, jx, kx), False)


def write_1d(path, a, mtype: int = MTYPE_FLOAT64) -> None:
    """dacdef1d + one write + close (the model packages' static outputs)."""
    with dacdef1d(path, np.asarray(a).size, mtype) as w:
        w.write(a)


class DacFile:
    """A DAC data file read whole: ``mtype``, ``dims`` (the extents without
    the time axis), ``unlimited`` and ``records`` (shape (n,) + dims reversed,
    i.e. C order with x fastest)."""

    def __init__(self, path):
        self.path = Path(path)
        raw = self.path.read_bytes()
        recs = []
        pos = 0
        while pos < len(raw):
            if pos + 4 > len(raw):
                raise DacError(f"{self.path.name}: truncated record marker at {pos}")
            (n,) = struct.unpack_from("<i", raw, pos)
            end = pos + 4 + n
            if n < 0 or end + 4 > len(raw):
                raise DacError(f"{self.path.name}: truncated record at {pos}")
            (n2,) = struct.unpack_from("<i", raw, end)
            if n2 != n:
                raise DacError(f"{self.path.name}: record markers differ at {pos}")
            recs.append(raw[pos + 4:end])
            pos = end + 4
        if len(recs) < 5:
            raise DacError(f"{self.path.name}: header incomplete")

        def one_int(b):
            if len(b) != 4:
                raise DacError(f"{self.path.name}: header record of {len(b)} bytes")
            return struct.unpack("<i", b)[0]

        # dacopnr*.f checks: byte-order probe and version
        if one_int(recs[0]) != 1:
            raise DacError(f"{self.path.name}: endian different")
        if one_int(recs[1]) != 0:
            raise DacError(f"{self.path.name}: version different")
        self.mtype = one_int(recs[2])
        if self.mtype not in _DTYPE:
            raise DacError(f"{self.path.name}: mtype {self.mtype}")
        rank = one_int(recs[3])
        ext = struct.unpack("<%di" % (len(recs[4]) // 4), recs[4])
        if len(ext) != rank:
            raise DacError(f"{self.path.name}: rank {rank} with {len(ext)} extents")
        self.unlimited = rank > 0 and ext[-1] == -1
        self.dims = tuple(ext[:-1]) if self.unlimited else tuple(ext)
        dt = _DTYPE[self.mtype]
        count = int(np.prod(self.dims)) if self.dims else 1
        data = []
        for k, b in enumerate(recs[5:]):
            if len(b) != count * dt.itemsize:
                raise DacError(f"{self.path.name}: data record {k} of {len(b)} bytes")
            data.append(np.frombuffer(b, dtype=dt).reshape(tuple(reversed(self.dims))))
        self.records = (np.stack(data) if data else
                        np.zeros((0,) + tuple(reversed(self.dims)), dtype=dt))

    @property
    def nx(self) -> int:
        return len(self.records)

    def last(self) -> np.ndarray:
        """The last record: what a restart (mcont=1) reads, the reference
        reading records until the end of the file."""
        if not len(self.records):
            raise DacError(f"{self.path.name}: no data record")
        return self.records[-1].copy()


def dacopnr(path, rank: int | None = None) -> DacFile:
    """cansio/dacopnr{0,1,2,3,4}s.f and dacopnr1d.f: open and check a file
    (with the rank check of the *s readers when ``rank`` is given: the number
    of array extents, the time axis not counted)."""
    f = DacFile(path)
    if rank is not None and len(f.dims) != rank:
        raise DacError(f"{f.path.name}: dimension different ({len(f.dims)} != {rank})")
    return f


# ---- params.txt -------------------------------------------------------------

def _e20_13(v: float) -> str:
    """Fortran E20.13 of a double: ' 0.ddddddddddddd E+xx' (mantissa in
    [0.1, 1), two-digit exponent, three digits beyond 99)."""
    v = float(v)
    if v == 0.0:
        s = "0.0000000000000E+00"
    elif not np.isfinite(v):
        s = "Infinity" if v > 0 else ("-Infinity" if v < 0 else "NaN")
        return s.rjust(20)
    else:
        m, e = "%.12e" % abs(v), 0
        # scientific d.dddddddddddde+xx -> 0.ddddddddddddd, exponent + 1
        digits, ex = m.split("e")
        d = digits.replace(".", "")
        e = int(ex) + 1
        # rounding to 13 significant digits can carry into a new digit
        if len(d) > 13:
            d = d[:13]
        es = "%+03d" % e if abs(e) < 100 else "%+04d" % e
        s = "0." + d + ("E" + es if abs(e) < 100 else es)
        if v < 0:
            s = "-" + s
    return s.rjust(20)


class DacParams:
    """params.txt writer (dacdefparam / dacputparam*) and reader
    (dacgetparam*).  Lines are appended as they are put."""

    def __init__(self, path, mode: str = "w"):
        self.path = Path(path)
        self._f = open(self.path, mode)

    def _line(self, mtype: int, name: str, value: str) -> None:
        # format('#dac ',i4,a32,' ',...): a32 right-justifies a shorter name
        self._f.write("#dac " + ("%4d" % mtype) + name[:32].rjust(32) + " " + value + "\n")
        self._f.flush()

    def puti(self, name: str, v: int) -> None:
        """dacputparami: type 4, i20."""
        self._line(4, name, ("%d" % int(v)).rjust(20))

    def putd(self, name: str, v: float) -> None:
        """dacputparamd: type 5, e20.13."""
        self._line(5, name, _e20_13(v))

    def putr(self, name: str, v: float) -> None:
        """dacputparam (real*4 value): type 5, e20.13 of the widened value."""
        self._line(5, name, _e20_13(float(np.float32(v))))

    def putc(self, name: str, v: str) -> None:
        """dacputparamc: type 2, a20."""
        self._line(2, name, str(v)[:20].rjust(20))

    def close(self) -> None:
        if not self._f.closed:
            self._f.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def read_params(path) -> dict:
    """All '#dac' lines of a parameter file as {name: value} (int for type 4,
    float for type 5, str for type 2), as the IDL reader dacgetparam splits
    them."""
    out = {}
    for line in Path(path).read_text().splitlines():
        if not line.startswith("#dac"):
            continue
        parts = line.split()
        if len(parts) < 4:
            continue
        mtype, name = int(parts[1]), parts[2]
        if mtype == 4:
            out[name] = int(parts[3])
        elif mtype == 5:
            out[name] = float(parts[3].replace("D", "E"))
        else:
            out[name] = line[line.index(name) + len(name):].strip()
    return out
