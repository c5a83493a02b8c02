"""The rational-function generator (milc_qcd_gb300/remez.py) against the
reference's own generator output: for every function of MILC's sample
rational file for the HISQ RHMC regression (read back from the fixture),
the generated approximation of the same degree on the same interval
[1e-15, 90] reaches the same maximum relative error (within a few per
cent) with its poles within 1 % of MILC's; the file writer round-trips
through the reader; the Naik epsilon series matches the value the
reference's calc_eps_naik.pl script prints for the config's charm mass."""
import numpy as np
import pytest

import rhmc_sample as R

pytest.importorskip("scipy")

TAGS = ("MD", "GR", "FA")
# y/z/m of the sample file's functions (rationals.sample.su3_rhmc_hisq)
SPECS = {0: ((-2, -1, 3, 0), (4, 4, 4, 4), (0.0018, 0.018, 0.2, 1.0)),
         1: ((-1, 0, 0, 0), (4, 4, 4, 4), (0.2, 1.0, 1.0, 1.0))}
SIGN = {"MD": 1, "GR": -1, "FA": 1}
ZSCALE = {"MD": 1, "GR": 2, "FA": 2}


def _spec(ipf, tag):
    y, z, m = SPECS[ipf]
    return tuple(SIGN[tag] * v for v in y), tuple(ZSCALE[tag] * v for v in z), m


@pytest.mark.parametrize("ipf", [0, 1])
@pytest.mark.parametrize("tag", TAGS)
def test_generator_matches_milc_sample(ipf, tag):
    from milc_qcd_gb300.remez import rational_function, max_rel_error
    from milc_qcd_gb300.rhmc import RationalFunction
    d = R.load()
    res, pole = d["rational"][ipf][tag]
    y, z, m = _spec(ipf, tag)
    milc = RationalFunction(y, z, m, len(res) - 1, res, pole)
    ours = rational_function(y, z, m, 1e-15, 90.0, len(res) - 1)
    e_milc, e_ours = max_rel_error(milc, 1e-15, 90.0, 200000), max_rel_error(ours, 1e-15, 90.0, 200000)
    # the minimax approximation is unique: the reference's error to 0.1 %
    assert abs(e_ours - e_milc) < 1e-3 * e_milc, (e_ours, e_milc)
    assert np.allclose(sorted(ours.pole[1:]), sorted(milc.pole[1:]), rtol=1e-3)
    assert abs(ours.res[0] - milc.res[0]) < 1e-4 * abs(milc.res[0])


def test_remez_polish_equioscillates():
    """The polished error alternates in sign at 2n+2 points with equal
    magnitude (the Chebyshev alternation that characterises the minimax)."""
    from milc_qcd_gb300.remez import rational_function, target, _alternant
    rf = rational_function((-1, 0, 0, 0), (2, 4, 4, 4), (0.05, 1, 1, 1), 1e-10, 50.0, 8)
    t = np.linspace(np.log(1e-10), np.log(50.0), 200000)
    x = np.exp(t)
    e = (rf.res[0] + sum(r / (x + p) for r, p in zip(rf.res[1:], rf.pole[1:]))) / target(rf.y, rf.z, rf.m)(x) - 1
    idx = _alternant(t, e, 2 * 8 + 2)
    assert len(idx) == 18
    assert np.all(np.sign(e[idx][1:]) != np.sign(e[idx][:-1]))
    peaks = np.abs(e[idx])
    assert peaks.max() - peaks.min() < 1e-3 * peaks.max()


def test_file_round_trip():
    from milc_qcd_gb300.remez import rational_function, format_rhmc_params
    from milc_qcd_gb300.rhmc import parse_rhmc_params
    fns = [rational_function((-1, 0, 0, 0), (z, 4, 4, 4), (0.1, 1, 1, 1), 1e-8, 60.0, 6) for z in (4, 8, 8)]
    text = format_rhmc_params([(0.0, fns[0], fns[1], fns[2])])
    back = parse_rhmc_params(text, 1)[0]
    for a, b in zip((back.MD, back.GR, back.FA), fns):
        assert a.order == b.order and np.allclose(a.res, b.res, rtol=1e-15) and np.allclose(a.pole, b.pole, rtol=1e-15)


def test_eps_naik():
    from milc_qcd_gb300.remez import eps_naik
    m = 0.432
    want = -27 / 40 * m ** 2 + 327 / 1120 * m ** 4 - 15607 / 268800 * m ** 6 - 73697 / 3942400 * m ** 8
    assert abs(eps_naik(m) - want) < 1e-15
    assert -0.13 < eps_naik(m) < -0.11
