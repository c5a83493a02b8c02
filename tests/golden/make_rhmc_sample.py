"""Fixture from MILC's shipped HISQ RHMC regression (6^4, one trajectory).

ks_imp_rhmc/test/su3_rhmc_hisq.2.sample-in (double precision build,
INT_3G1F, 2+1 flavours, 4 pseudofermion fields) starts from
binary_samples/lat.sample.l6666.hisq and the rational functions in
ks_imp_rhmc/test/rationals.sample.su3_rhmc_hisq.  This script reads the
lattice (MILC's binary format v5 of generic/io_lat4.c: 96-byte header with
magic 20103, dims, time stamp, order, and the sum29/sum31 checksums, then
float32 su3_matrix[4] per site in lexicographic order; checksums verified),
puts the sites in MILC's even-first order, parses the rational functions
and stores both in rhmc_hisq_6666.npz.  The run parameters and MILC's
printed results are constants of tests/rhmc_sample.py.

Run:  python tests/golden/make_rhmc_sample.py [reference root]
"""
import ctypes
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

def _reference():
    """The reference tree ($MILC_REFERENCE_DIR, or the one oracle/_ref was built from)."""
    from oracle.oracle import reference_tree
    ref = reference_tree()
    if not ref:
        raise SystemExit("reference tree not found: set MILC_REFERENCE_DIR")
    return ref


DEFAULT = None


def read_milc_lattice(path):
    data = open(path, "rb").read()
    magic = struct.unpack("<i", data[:4])[0]
    if magic != 20103:
        raise ValueError("%s: not a little-endian MILC v5 lattice (magic %d)" % (path, magic))
    dims = struct.unpack("<4i", data[4:20])
    order = struct.unpack("<i", data[84:88])[0]
    if order != 0:
        raise ValueError("%s: only serial-order files are read" % path)
    sum29, sum31 = struct.unpack("<II", data[88:96])
    words = np.frombuffer(data[96:], dtype="<u4").astype(np.uint64)
    k = np.arange(words.size, dtype=np.uint64)

    def rot(r):
        return ((words << r) | (words >> ((np.uint64(32) - r) % np.uint64(32)))) & np.uint64(0xFFFFFFFF)

    c29 = int(np.bitwise_xor.reduce(rot(k % np.uint64(29))))
    c31 = int(np.bitwise_xor.reduce(rot(k % np.uint64(31))))
    if (c29, c31) != (sum29, sum31):
        raise ValueError("%s: checksum mismatch" % path)
    V = int(np.prod(dims))
    return tuple(dims), np.frombuffer(data[96:], dtype="<f4").reshape(V, 4, 18)


def main(ref=DEFAULT):
    ref = ref or _reference()
    from milc_qcd_gb300 import _lib
    from milc_qcd_gb300.rhmc import load_rhmc_params
    dims, lat = read_milc_lattice(os.path.join(ref, "binary_samples", "lat.sample.l6666.hisq"))
    lib = _lib.load()
    d4 = (ctypes.c_int * 4)(*dims)
    V = lat.shape[0]
    perm = np.zeros(V, dtype=np.int64)
    for r in range(V):
        c = (r % dims[0], (r // dims[0]) % dims[1], (r // (dims[0] * dims[1])) % dims[2],
             r // (dims[0] * dims[1] * dims[2]))
        perm[r] = lib.mks_site_index(d4, (ctypes.c_int * 4)(*c))
    U = np.zeros_like(lat)
    U[perm] = lat
    P = load_rhmc_params(os.path.join(ref, "ks_imp_rhmc", "test", "rationals.sample.su3_rhmc_hisq"), 4)
    out = dict(dims=np.array(dims, dtype=np.int32), lat=U, naik_eps=np.array([p.naik_term_epsilon for p in P]))
    for i, p in enumerate(P):
        for tag in ("MD", "GR", "FA"):
            f = getattr(p, tag)
            out["%s_res_%d" % (tag, i)] = np.array(f.res)
            out["%s_pole_%d" % (tag, i)] = np.array(f.pole)
    path = os.path.join(HERE, "rhmc_hisq_6666.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(*sys.argv[1:])
