"""MILC's HISQ RHMC regression on 6^4 (double precision), as data.

Run parameters: ks_imp_rhmc/test/su3_rhmc_hisq.2.sample-in.  Printed
results: ks_imp_rhmc/test/su3_rhmc_hisq.2.sample-out (line numbers below);
tolerances from su3_rhmc_hisq.2.errtol where it gives them.  The lattice
and rational functions are in tests/golden/rhmc_hisq_6666.npz
(tests/golden/make_rhmc_sample.py).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "rhmc_hisq_6666.npz")

DIMS = (6, 6, 6, 6)
ISEED = 86658
BETA = 7.4
U0 = 0.89
DYN_FLAVORS = (2, 1)                   # dyn_mass .0018 .018, dyn_flavors 2 1
N_PSEUDO = 4
EPSILON = 0.02                          # microcanonical_time_step
STEPS = 10                              # steps_per_trajectory
INT_ALG = "3G1F"                        # ks_imp_rhmc/Make_template:203 (HISQ_OPTIONS)
# cgresid_md_fa_gr (residuals, not squared) and max_multicg_md_fa_gr, per field
RESID_MD = (5e-4, 5e-6, 5e-6, 5e-6)
RESID_FA = (1e-4, 1e-6, 1e-6, 1e-6)
RESID_GR = (1e-4, 1e-6, 1e-6, 1e-6)
MAX_CG = 2500
NRESTART = 5

# su3_rhmc_hisq.2.sample-out
PLAQ_START = (1.8403954419120214e+00, 1.8597505785271828e+00)                   # :492 CHECK PLAQ
GRSOURCE_SUMS = (1.9636750556e+03, 1.9027332579e+03, 1.9328576806e+03, 1.9363357347e+03)  # :526-532
ACTION_START = (1.91689566918234e+04, -8.03775303465063e+01, 7.73560172845149e+03)  # :539 g, h, f
ACTION_END = (1.89814618171498e+04, 1.10640260690474e+02, 7.73207879686826e+03)     # :597
DELTA_S = -1.521986e-05                                                           # :599
DELTA_S_TOL = 0.02                                                                # errtol: ACCEPT
PLAQ_END = (1.8590262183356623, 1.8640148066269224)                               # :600
PLAQ_END_TOL = (8e-07, 2e-06)                                                     # errtol: PLAQ


def load():
    d = np.load(FIXTURE)
    out = {k: d[k] for k in d.files}
    rat = []
    for i in range(N_PSEUDO):
        rat.append({tag: (out["%s_res_%d" % (tag, i)], out["%s_pole_%d" % (tag, i)]) for tag in ("MD", "GR", "FA")})
    out["rational"] = rat
    return out


def nflavors():
    return sum(DYN_FLAVORS)
