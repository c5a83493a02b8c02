"""Fixture from MILC's own shipped test vectors (asqtad, 8^4 lattice).

MILC's check programs ks_imp_utilities/check_ks_invert.c and
check_fermion_force.c (run by ks_imp_utilities/test/Makefile) read
binary_samples/lat.sample.l8 (u0 = 0.502), binary_samples/
ksvector.src.sample.l8, and compare against

  ksvector.ans.MdaggerMinv.sample.l8  (M^dag M)^-1 src, both parities, mass 0.1
  ksvector.ans.Minv.sample.l8         M^-1 src, mass 0.1
  colormatrix.mom.sample.l8           uncompressed force, eps = 1, residue 1
  fat.l8 / long.l8                    the asqtad fat and long links (phases in)

This script reads those SciDAC files (checksums verified), puts every site
into MILC's even-first order (the package's host geometry) and writes
milc_sample_l8.npz: the lattice, source and both solutions whole (float32,
as stored), and the fat, long and force fields on a fixed subset of 512
sites to keep the fixture small.

Run:  python tests/golden/make_milc_samples.py [binary_samples folder]
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import scidac  # noqa: E402

DEFAULT = None  # the reference tree's binary_samples ($MILC_REFERENCE_DIR, or oracle/_ref's source tree)
NSUB = 512


def milc_order(dims):
    """perm[r] = MILC index of the site with lexicographic rank r."""
    from milc_qcd_gb300 import _lib
    lib = _lib.load()
    d4 = (ctypes.c_int * 4)(*dims)
    V = int(np.prod(dims))
    perm = np.zeros(V, dtype=np.int64)
    for r in range(V):
        x = r % dims[0]
        y = (r // dims[0]) % dims[1]
        z = (r // (dims[0] * dims[1])) % dims[2]
        t = r // (dims[0] * dims[1] * dims[2])
        perm[r] = lib.mks_site_index(d4, (ctypes.c_int * 4)(x, y, z, t))
    return perm


def main(folder=DEFAULT):
    if not folder:
        from oracle.oracle import reference_tree
        ref = reference_tree()
        if not ref:
            raise SystemExit("reference tree not found: set MILC_REFERENCE_DIR")
        folder = os.path.join(ref, "binary_samples")
    lat, info = scidac.read_field(os.path.join(folder, "lat.sample.l8"))
    dims = tuple(info["dims"])
    perm = milc_order(dims)
    V = len(perm)

    def load(name):
        f, _ = scidac.read_field(os.path.join(folder, name))
        out = np.zeros_like(f)
        out[perm] = f
        return out.astype(np.float32)

    rng = np.random.default_rng(20050216)
    sub = np.sort(rng.choice(V, NSUB, replace=False)).astype(np.int32)
    out = dict(
        dims=np.array(dims, dtype=np.int32),
        lat=load("lat.sample.l8"),
        src=load("ksvector.src.sample.l8")[:, 0],
        ans_mdagm=load("ksvector.ans.MdaggerMinv.sample.l8")[:, 0],
        ans_m=load("ksvector.ans.Minv.sample.l8")[:, 0],
        sub=sub,
        fat_sub=load("fat.l8")[sub],
        long_sub=load("long.l8")[sub],
        mom_sub=load("colormatrix.mom.sample.l8")[sub],
    )
    path = os.path.join(HERE, "milc_sample_l8.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(*sys.argv[1:])
