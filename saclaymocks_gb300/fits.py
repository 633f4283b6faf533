"""Minimal FITS reader/writer for the file formats on the SaclayMocks hot path.

The reference reads and writes FITS through ``fitsio``:

* ``etc/params.fits`` (BINTABLE z, a, b, c), ``etc/p1dmiss_z*.fits`` (k, P1Dmiss[RSD]),
  ``etc/dgrowth.fits`` (Z, dD/dz) are read by ``util.InterpFitsTable``
  (py/SaclayMocks/util.py:300-314) and ``bin/merge_spectra.py:105-118``;
* ``box-{i}.fits`` / ``eta_zz-{i}.fits`` are written one x-plane per file as a float32
  primary image with keys DX, DY, DZ, NX, NY, NZ (+ sigma, seed on file 0)
  by ``FFTandStore`` (bin/make_boxes.py:110-117);
* ``spectra-*.fits.gz`` / ``spectra_merged-*.fits.gz`` hold a METADATA table plus
  float32 image HDUs (bin/make_spectra.py:566-597, bin/merge_spectra.py:385-406).

Only what those formats use is supported: images of BITPIX 8/16/32/64/-32/-64 and
binary tables with scalar or fixed-repeat columns of types L, B, I, J, K, E, D, A.
Files ending in ``.gz`` are transparently (de)compressed.  This module is host-side
file plumbing; it holds no numerics.
"""
from __future__ import annotations

import gzip
import os
from dataclasses import dataclass, field

import numpy as np

BLOCK = 2880

_BITPIX_DTYPE = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}
_DTYPE_BITPIX = {np.dtype(v).newbyteorder("=").str[1:]: k for k, v in _BITPIX_DTYPE.items()}
_TFORM_DTYPE = {"L": "i1", "B": "u1", "I": ">i2", "J": ">i4", "K": ">i8",
                "E": ">f4", "D": ">f8"}


class FitsError(ValueError):
    """Raised for a malformed or unsupported FITS stream."""


@dataclass
class HDU:
    header: dict
    data: object = None
    comments: dict = field(default_factory=dict)

    @property
    def name(self) -> str:
        return str(self.header.get("EXTNAME", "")).strip()


# ----------------------------------------------------------------------------- parsing
def _parse_value(raw: str):
    raw = raw.strip()
    if not raw:
        return None
    if raw.startswith("'"):
        # string: '' is an escaped quote, trailing blanks are not significant
        out, i = [], 1
        while i < len(raw):
            ch = raw[i]
            if ch == "'":
                if i + 1 < len(raw) and raw[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(ch)
            i += 1
        return "".join(out).rstrip()
    val = raw.split("/")[0].strip()
    if val == "T":
        return True
    if val == "F":
        return False
    try:
        return int(val)
    except ValueError:
        pass
    try:
        return float(val.replace("D", "E"))
    except ValueError:
        return val


def _read_header(buf: bytes, pos: int):
    header, comments = {}, {}
    while True:
        if pos + BLOCK > len(buf):
            raise FitsError("truncated FITS header")
        block = buf[pos:pos + BLOCK]
        pos += BLOCK
        for j in range(0, BLOCK, 80):
            card = block[j:j + 80].decode("ascii", "replace")
            key = card[:8].strip()
            if key == "END":
                return header, comments, pos
            if key == "HIERARCH":
                body = card[9:]
                if "=" in body:
                    k, v = body.split("=", 1)
                    header[k.strip().upper()] = _parse_value(v)
                continue
            if card[8:10] == "= ":
                val = _parse_value(card[10:])
                header[key] = val
                if "/" in card[10:] and not card[10:].strip().startswith("'"):
                    comments[key] = card[10:].split("/", 1)[1].strip()


def _data_bytes(h: dict) -> int:
    naxis = int(h.get("NAXIS", 0))
    if naxis == 0:
        return 0
    n = 1
    for i in range(1, naxis + 1):
        n *= int(h[f"NAXIS{i}"])
    n = n * abs(int(h["BITPIX"])) // 8
    return int(h.get("GCOUNT", 1)) * (int(h.get("PCOUNT", 0)) + n)


def _table_dtype(h: dict) -> np.dtype:
    names, formats = [], []
    for i in range(1, int(h["TFIELDS"]) + 1):
        name = str(h.get(f"TTYPE{i}", f"col{i}")).strip()
        tform = str(h[f"TFORM{i}"]).strip()
        digits = "".join(ch for ch in tform if ch.isdigit())
        code = tform[len(digits):][:1]
        rep = int(digits) if digits else 1
        if code == "A":
            formats.append(f"S{rep}")
        elif code in _TFORM_DTYPE:
            base = _TFORM_DTYPE[code]
            formats.append(base if rep == 1 else (base, (rep,)))
        else:
            raise FitsError(f"unsupported TFORM {tform!r}")
        names.append(name)
    dt = np.dtype({"names": names, "formats": formats})
    if dt.itemsize != int(h["NAXIS1"]):
        raise FitsError("table row size does not match NAXIS1")
    return dt


def _load_bytes(path: str) -> bytes:
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    return raw


def read_fits(path: str) -> list:
    """Return every HDU of ``path`` as :class:`HDU` (image -> ndarray in C order,
    table -> structured ndarray, no data -> None)."""
    buf = _load_bytes(path)
    hdus, pos = [], 0
    while pos + BLOCK <= len(buf):
        if not buf[pos:pos + 80].strip(b" \x00"):
            break
        h, c, pos = _read_header(buf, pos)
        nbytes = _data_bytes(h)
        raw = buf[pos:pos + nbytes]
        if len(raw) < nbytes:
            raise FitsError("truncated FITS data")
        xt = str(h.get("XTENSION", "")).strip()
        data = None
        if xt == "BINTABLE":
            dt = _table_dtype(h)
            data = np.frombuffer(raw, dtype=dt, count=int(h["NAXIS2"])).copy()
        elif int(h.get("NAXIS", 0)) > 0:
            shape = tuple(int(h[f"NAXIS{i}"]) for i in range(int(h["NAXIS"]), 0, -1))
            data = np.frombuffer(raw, dtype=_BITPIX_DTYPE[int(h["BITPIX"])],
                                 count=int(np.prod(shape))).reshape(shape)
            bscale, bzero = h.get("BSCALE", 1), h.get("BZERO", 0)
            data = data.astype(data.dtype.newbyteorder("="))
            if bscale != 1 or bzero != 0:
                data = data * bscale + bzero
        hdus.append(HDU(h, data, c))
        pos += (nbytes + BLOCK - 1) // BLOCK * BLOCK
    return hdus


def _find(hdus: list, ext):
    if isinstance(ext, int):
        return hdus[ext]
    for h in hdus:
        if h.name.upper() == str(ext).upper():
            return h
    raise KeyError(f"no HDU named {ext!r}")


def read(path: str, ext=None):
    """``fitsio.read`` subset: data of HDU ``ext`` (default: first HDU holding data)."""
    hdus = read_fits(path)
    if ext is None:
        for h in hdus:
            if h.data is not None:
                return h.data
        raise FitsError("no data in file")
    return _find(hdus, ext).data


def read_header(path: str, ext=0) -> dict:
    return dict(_find(read_fits(path), ext).header)


def read_table_columns(path: str, ext=1) -> dict:
    """BINTABLE as ``{column: native-endian ndarray}``."""
    tab = read(path, ext)
    return {n: np.asarray(tab[n]).astype(tab.dtype[n].base.newbyteorder("="))
            for n in tab.dtype.names}


# ----------------------------------------------------------------------------- writing
def _card(key: str, value, comment: str = "") -> bytes:
    if isinstance(value, (bool, np.bool_)):
        v = "T" if value else "F"
        s = f"{key:<8}= {v:>20}"
    elif isinstance(value, (int, np.integer)):
        s = f"{key:<8}= {int(value):>20d}"
    elif isinstance(value, (float, np.floating)):
        s = f"{key:<8}= {repr(float(value)).upper():>20}"
    elif value is None:
        s = f"{key:<8}="
    else:
        txt = str(value).replace("'", "''")
        s = f"{key:<8}= '{txt:<8}'"
    if comment:
        s += " / " + comment
    s = s[:80]
    return s.ljust(80).encode("ascii")


def _pad(b: bytes, fill: bytes) -> bytes:
    return b + fill * ((-len(b)) % BLOCK)


def _image_hdu(arr: np.ndarray, header: dict, primary: bool, extname=None) -> bytes:
    arr = np.ascontiguousarray(arr)
    key = arr.dtype.newbyteorder("=").str[1:]
    if key not in _DTYPE_BITPIX:
        raise FitsError(f"unsupported image dtype {arr.dtype}")
    bitpix = _DTYPE_BITPIX[key]
    cards = [_card("SIMPLE", True) if primary else _card("XTENSION", "IMAGE"),
             _card("BITPIX", bitpix), _card("NAXIS", arr.ndim)]
    for i, n in enumerate(arr.shape[::-1], 1):
        cards.append(_card(f"NAXIS{i}", int(n)))
    if primary:
        cards.append(_card("EXTEND", True))
    else:
        cards += [_card("PCOUNT", 0), _card("GCOUNT", 1)]
    if extname:
        cards.append(_card("EXTNAME", extname))
    for k, v in (header or {}).items():
        cards.append(_card(k.upper()[:8], v))
    cards.append(b"END".ljust(80))
    data = arr.astype(_BITPIX_DTYPE[bitpix], copy=False).tobytes()
    return _pad(b"".join(cards), b" ") + _pad(data, b"\x00")


def _table_hdu(columns: dict, header: dict, extname=None) -> bytes:
    names = list(columns)
    cols = [np.asarray(columns[n]) for n in names]
    nrow = len(cols[0]) if cols else 0
    rev = {v: k for k, v in _TFORM_DTYPE.items() if k != "L"}
    fmts, dts = [], []
    for n, c in zip(names, cols):
        if len(c) != nrow:
            raise FitsError("table columns differ in length")
        rep = int(np.prod(c.shape[1:])) if c.ndim > 1 else 1
        if c.dtype.kind in "SU":
            c = c.astype("S")
            fmts.append(f"{c.dtype.itemsize}A")
            dts.append((n, c.dtype.str))
            continue
        be = c.dtype.newbyteorder(">").str
        if c.dtype.kind == "b":
            be, code = "i1", "L"
        elif be in rev:
            code = rev[be]
        elif c.dtype.kind == "u" and c.dtype.itemsize == 1:
            be, code = "u1", "B"
        else:
            raise FitsError(f"unsupported column dtype {c.dtype}")
        fmts.append(f"{rep}{code}" if rep > 1 else code)
        dts.append((n, be, c.shape[1:]) if rep > 1 else (n, be))
    rec = np.zeros(nrow, dtype=dts)
    for n, c in zip(names, cols):
        rec[n] = c.astype("S") if c.dtype.kind == "U" else c
    cards = [_card("XTENSION", "BINTABLE"), _card("BITPIX", 8), _card("NAXIS", 2),
             _card("NAXIS1", rec.dtype.itemsize), _card("NAXIS2", nrow),
             _card("PCOUNT", 0), _card("GCOUNT", 1), _card("TFIELDS", len(names))]
    for i, (n, f) in enumerate(zip(names, fmts), 1):
        cards += [_card(f"TTYPE{i}", n), _card(f"TFORM{i}", f)]
    if extname:
        cards.append(_card("EXTNAME", extname))
    for k, v in (header or {}).items():
        cards.append(_card(k.upper()[:8], v))
    cards.append(b"END".ljust(80))
    return _pad(b"".join(cards), b" ") + _pad(rec.tobytes(), b"\x00")


class FitsWriter:
    """Sequential writer: ``w.image(arr, header)`` / ``w.table(cols, header)``; the first
    image goes to the primary HDU, a first table is preceded by an empty primary."""

    def __init__(self, path: str):
        self.path = path
        self._parts: list = []

    def image(self, arr, header=None, extname=None):
        self._parts.append(_image_hdu(np.asarray(arr), header, not self._parts, extname))
        return self

    def table(self, columns: dict, header=None, extname=None):
        if not self._parts:
            self._parts.append(_empty_primary())
        self._parts.append(_table_hdu(columns, header, extname))
        return self

    def close(self):
        blob = b"".join(self._parts)
        tmp = self.path + ".part"
        if self.path.endswith(".gz"):
            with gzip.open(tmp, "wb", compresslevel=1) as f:
                f.write(blob)
        else:
            with open(tmp, "wb") as f:
                f.write(blob)
        os.replace(tmp, self.path)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is None:
            self.close()


def _empty_primary() -> bytes:
    cards = [_card("SIMPLE", True), _card("BITPIX", 16), _card("NAXIS", 0),
             _card("EXTEND", True), b"END".ljust(80)]
    return _pad(b"".join(cards), b" ")


def write_image(path: str, arr, header=None):
    FitsWriter(path).image(arr, header).close()
