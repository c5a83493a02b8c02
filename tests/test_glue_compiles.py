"""The MILC-side binding (milc_qcd_gb300/milc_glue/mks_milc_glue.c) compiles
against MILC's headers, and so do the MILC files the USE_*_GPU macro swaps
touch.  Needs the reference tree; skipped elsewhere."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle.oracle import reference_tree

REF = reference_tree() or "<no reference tree>"
pytestmark = pytest.mark.skipif(reference_tree() is None, reason="reference tree not present")

FLAGS = ["-fsyntax-only", "-std=gnu99", "-w", "-DMILC_PRECISION=2", "-DFN", "-DHMC", "-DHISQ_FF_MULTI_WRAPPER",
         "-DSINGLE", "-DINT_ALG=INT_3G1F", "-DKS_MULTICG=HYBRID", "-DKS_MULTIFF=FNMAT", "-DFEWSUMS",
         "-DDBLSTORE_FN", "-DUSE_CG_GPU", "-DUSE_FL_GPU", "-DUSE_FF_GPU",
         "-include", os.path.join(ROOT, "milc_qcd_gb300", "milc_glue", "mks_milc_alloc.h")]


def _inc(tmp_path):
    inc = tmp_path / "inc"
    inc.mkdir()
    (inc / "quark_action.h").write_text('#include "%s/generic_ks/imp_actions/hisq/hisq_u3_action.h"\n' % REF)
    (inc / "gauge_action.h").write_text('#include "%s/generic/imp_actions/symanzik_1loop_hisq_action.h"\n' % REF)
    return ["-I" + str(inc), "-I" + REF + "/ks_imp_rhmc", "-I" + REF + "/include", "-I" + REF + "/generic_ks",
            "-I" + os.path.join(ROOT, "include")]


def test_glue_compiles_for_asqtad(tmp_path):
    src = os.path.join(ROOT, "milc_qcd_gb300", "milc_glue", "mks_milc_glue.c")
    inc = _inc(tmp_path)
    (tmp_path / "inc" / "quark_action.h").write_text('#include "%s/generic_ks/imp_actions/asqtad_action.h"\n' % REF)
    (tmp_path / "inc" / "gauge_action.h").write_text('#include "%s/generic/imp_actions/symanzik_1loop_action.h"\n' % REF)
    flags = [f for f in FLAGS if f != "-DHISQ_FF_MULTI_WRAPPER"]
    r = subprocess.run(["gcc"] + flags + ["-DUSE_GF_GPU"] + inc + [src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_glue_compiles_with_gpu_gauge_side(tmp_path):
    src = os.path.join(ROOT, "milc_qcd_gb300", "milc_glue", "mks_milc_glue.c")
    r = subprocess.run(["gcc"] + FLAGS + ["-DUSE_GF_GPU"] + _inc(tmp_path) + [src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.parametrize("src", [
    os.path.join(ROOT, "milc_qcd_gb300", "milc_glue", "mks_milc_glue.c"),
    REF + "/generic_ks/fermion_links_hisq_load_milc.c",
    REF + "/generic_ks/fn_links_milc.c",
    REF + "/generic_ks/fermion_links_from_site.c",
    REF + "/generic_ks/d_congrad5_fn.c",
    REF + "/generic_ks/ks_multicg.c",
    REF + "/generic_ks/mat_invert.c",
])
def test_compiles(tmp_path, src):
    r = subprocess.run(["gcc"] + FLAGS + _inc(tmp_path) + [src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
