"""Minimal SciDAC/LIME reader for MILC's serial single-file fields.

Test infrastructure: used only by make_milc_samples.py to turn the
reference's binary sample files into fixtures.

Format (as MILC writes it through QIO, e.g. generic/io_scidac.c):
a LIME file is a sequence of records, each a 144-byte big-endian header
(magic 0x456789ab, version, flags, data length, 128-byte type string)
followed by the data padded to 8 bytes.  A field is stored as the records
``scidac-private-record-xml`` (datatype, precision, colors, datacount),
``scidac-record-xml`` (user string), ``scidac-binary-data`` (all sites in
lexicographic order x fastest, then y, z, t; big-endian reals; complex as
re, im; matrices row-major; `datacount` objects per site) and
``scidac-checksum`` (suma / sumb).

The checksum is the SciDAC one: for the site of lexicographic rank r,
c = crc32(site bytes); suma ^= rotl32(c, r mod 29); sumb ^= rotl32(c, r mod 31).
"""
import re
import struct
import zlib

import numpy as np

LIME_MAGIC = 0x456789AB


def lime_records(path):
    """List of (type, bytes) in file order."""
    data = open(path, "rb").read()
    out, off = [], 0
    while off + 144 <= len(data):
        magic, _ver, _flags, length = struct.unpack(">IHHQ", data[off:off + 16])
        if magic != LIME_MAGIC:
            raise ValueError("%s: bad LIME magic at offset %d" % (path, off))
        typ = data[off + 16:off + 144].split(b"\0")[0].decode()
        out.append((typ, data[off + 144:off + 144 + length]))
        off += 144 + ((length + 7) // 8) * 8
    return out


def _rotl(c, k):
    return ((c << k) | (c >> (32 - k))) & 0xFFFFFFFF if k else c


def scidac_checksum(binary, nsites):
    size = len(binary) // nsites
    suma = sumb = 0
    for r in range(nsites):
        c = zlib.crc32(binary[r * size:(r + 1) * size]) & 0xFFFFFFFF
        suma ^= _rotl(c, r % 29)
        sumb ^= _rotl(c, r % 31)
    return suma, sumb


def _tag(xml, name):
    m = re.search(r"<%s>([^<]*)</%s>" % (name, name), xml)
    return m.group(1).strip() if m else None


def read_field(path):
    """Returns (array, info).  array: float64, shape (V, datacount, ncomp)
    in lexicographic site order, ncomp = 18 (color matrix) or 6 (vector).
    The SciDAC checksum is verified."""
    recs = lime_records(path)
    types = [t for t, _ in recs]
    fxml = recs[types.index("scidac-private-file-xml")][1].decode(errors="replace")
    dims = [int(x) for x in _tag(fxml, "dims").split()]
    rxml = recs[types.index("scidac-private-record-xml")][1].decode(errors="replace")
    prec = _tag(rxml, "precision")
    datatype = _tag(rxml, "datatype")
    count = int(_tag(rxml, "datacount"))
    binary = recs[types.index("scidac-binary-data")][1]
    ck = recs[types.index("scidac-checksum")][1].decode(errors="replace")
    V = int(np.prod(dims))
    suma, sumb = scidac_checksum(binary, V)
    want = (int(_tag(ck, "suma"), 16), int(_tag(ck, "sumb"), 16))
    if (suma, sumb) != want:
        raise ValueError("%s: SciDAC checksum mismatch %08x %08x != %08x %08x" % ((path, suma, sumb) + want))
    dt = ">f4" if prec == "F" else ">f8"
    arr = np.frombuffer(binary, dtype=dt).astype(np.float64)
    ncomp = arr.size // (V * count)
    info = dict(dims=dims, precision=prec, datatype=datatype, datacount=count, checksum=want,
                user_record=recs[types.index("scidac-record-xml")][1].split(b"\0")[0].decode(errors="replace"),
                user_file=recs[types.index("scidac-file-xml")][1].split(b"\0")[0].decode(errors="replace"))
    return arr.reshape(V, count, ncomp), info
