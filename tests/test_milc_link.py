"""The drop-in, linked: MILC's own su3_rhmc_hisq application (ks_imp_rhmc),
compiled from the reference sources with the GPU object-list swap and
mks_milc_glue.c in place of the QUDA shims, links against
libmilc_ks_gb300.so with every symbol resolved
(milc_qcd_gb300/milc_glue/Makefile; the recipe of INTEGRATION.md).

The linked binary then runs MILC's own regression input
(ks_imp_rhmc/test/su3_rhmc_hisq.2.sample-in): MILC's set-up reads the
lattice and the rational functions and builds its path tables, and its
first fermion-link construction enters the library through the glue
(mks_init).  On a host without a GPU that call reports the missing device
and MILC terminates there; with a GPU the trajectory runs on it.  The GPU
host has no reference tree, so the binary is built and run here only.

Needs the reference tree; skipped elsewhere."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle.oracle import reference_tree

REF = reference_tree()
pytestmark = pytest.mark.skipif(REF is None, reason="reference tree not present")

LIB = os.path.join(ROOT, "milc_qcd_gb300", "libmilc_ks_gb300.so")


@pytest.fixture(scope="module")
def milc_app(tmp_path_factory):
    if not os.path.exists(LIB):
        from milc_qcd_gb300 import build
        build.build()
    out = tmp_path_factory.mktemp("milc_build")
    r = subprocess.run(["make", "-s", "-j%d" % (os.cpu_count() or 4), "-f",
                        os.path.join(ROOT, "milc_qcd_gb300", "milc_glue", "Makefile"), "REF=%s" % REF,
                        "OUT=%s" % out], capture_output=True, text=True)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    return str(out / "su3_rhmc_hisq_mks")


def test_su3_rhmc_hisq_links_against_the_library(milc_app):
    assert os.path.exists(milc_app)
    # the library is a direct dependency and every MILC-facing _gpu entry the
    # swap selects resolves to the glue, which calls the C ABI
    nm = subprocess.run(["nm", milc_app], capture_output=True, text=True).stdout
    defined = {l.split()[-1] for l in nm.splitlines() if len(l.split()) == 3 and l.split()[1] in "Tt"}
    for sym in ("ks_congrad_parity_gpu", "ks_congrad_block_parity_gpu", "ks_multicg_offset_field_gpu",
                "load_hisq_aux_links_gpu", "load_fatlonglinks_gpu", "eo_fermion_force_multi"):
        assert sym in defined, sym
    undefined = {l.split()[-1] for l in nm.splitlines() if l.split()[:1] == ["U"]}
    assert {"mks_init", "mks_ks_congrad_parity", "mks_ks_multicg_offset_field",
            "mks_fermion_force_multi_hisq"} <= undefined  # bound to the shared library at run time
    ldd = subprocess.run(["ldd", milc_app], capture_output=True, text=True).stdout
    assert "libmilc_ks_gb300.so" in ldd and "not found" not in ldd


def test_su3_rhmc_hisq_sample_input_reaches_the_library(milc_app, tmp_path):
    # the sample input names ../../binary_samples/... and a rationals file in the run folder
    (tmp_path / "binary_samples").symlink_to(os.path.join(REF, "binary_samples"))
    run = tmp_path / "a" / "b"
    run.mkdir(parents=True)
    (run / "rationals.sample.su3_rhmc_hisq").symlink_to(
        os.path.join(REF, "ks_imp_rhmc", "test", "rationals.sample.su3_rhmc_hisq"))
    with open(os.path.join(REF, "ks_imp_rhmc", "test", "su3_rhmc_hisq.2.sample-in")) as f:
        r = subprocess.run([milc_app], stdin=f, cwd=str(run), capture_output=True, text=True, timeout=300)
    out = r.stdout + r.stderr
    # MILC's own set-up ran: the lattice and the rational functions were read
    assert "MAKING PATH TABLES" in out, out[-3000:]
    assert "lat.sample.l6666.hisq" in out
    assert "rationals.sample.su3_rhmc_hisq" in out or "n_pseudo" in out
    if "mks_init" in out:
        # no GPU on this host: the glue's first library call reports it
        assert r.returncode != 0
    else:
        # a GPU host with the reference tree: the trajectory completed
        assert r.returncode == 0 and "RUNNING COMPLETED" in out, out[-3000:]
