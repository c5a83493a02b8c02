"""Rational functions for the 2+1+1 HISQ RHMC workload (48^3x96, masses
0.0012 / 0.0363 / 0.432), written in MILC's rational-file format by
milc_qcd_gb300.remez.

Fields (one pseudofermion each, on [1e-15, 90]; 16 poles for the light
pair, whose multi-shift solves dominate; 12 for the strange and 10 for the
charm field, where the approximation error is already ~1e-11 and more poles
only add near-cancelling pairs in double precision):
  0  light pair   MD (x+4 ml^2)^(-1/2)  GR (x+4 ml^2)^(1/4)  FA (x+4 ml^2)^(-1/4)
  1  strange      MD (x+4 ms^2)^(-1/4)  GR (x+4 ms^2)^(1/8)  FA (x+4 ms^2)^(-1/8)
  2  charm        as strange with mc and the Naik epsilon of am = 0.432

Run:  python milc_qcd_gb300/data/make_rationals.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from milc_qcd_gb300.remez import rational_function, format_rhmc_params, eps_naik  # noqa: E402

MASSES = {"light": 0.0012, "strange": 0.0363, "charm": 0.432}
LO, HI = 1e-15, 90.0
OUT = os.path.join(HERE, "rationals.hisq_2p1p1_ml0.0012_ms0.0363_mc0.432.txt")


ORDERS = {"light": 16, "strange": 12, "charm": 10}


def field(m, nf_num, order):
    """(x + 4 m^2)^(-nf/4) for MD, ^(nf/8) for GR, ^(-nf/8) for FA."""
    masses = (m, 1.0, 1.0, 1.0)
    md = rational_function((-nf_num, 0, 0, 0), (4, 4, 4, 4), masses, LO, HI, order)
    gr = rational_function((nf_num, 0, 0, 0), (8, 8, 8, 8), masses, LO, HI, order)
    fa = rational_function((-nf_num, 0, 0, 0), (8, 8, 8, 8), masses, LO, HI, order)
    return md, gr, fa


def main():
    fields = [(0.0,) + field(MASSES["light"], 2, ORDERS["light"]),
              (0.0,) + field(MASSES["strange"], 1, ORDERS["strange"]),
              (eps_naik(MASSES["charm"]),) + field(MASSES["charm"], 1, ORDERS["charm"])]
    with open(OUT, "w") as f:
        f.write("# 2+1+1 HISQ, ml = %g, ms = %g, mc = %g; generated by milc_qcd_gb300/data/make_rationals.py\n"
                % (MASSES["light"], MASSES["strange"], MASSES["charm"]))
        f.write(format_rhmc_params(fields) + "\n")
    for i, (eps, md, gr, fa) in enumerate(fields):
        print(i, "eps_naik %.6g" % eps, "max rel err MD %.2e GR %.2e FA %.2e" % (md.error, gr.error, fa.error))
    print("wrote", OUT)


if __name__ == "__main__":
    main()
