"""Constants against the reference's own: units and element tables
(PhysicalData.py), the PARAMS defaults (TMParams.py), and the DSF shift and
slope of the electrostatic embedding (Util.py DSF / DSF_Gradient).

tests/golden/make_golden_constants.py takes these from the reference tree.
The CUDA library's host copies of the unit and vdW tables in
tensormol_gb300/csrc/tm_api.cu are checked too, read from the source text.
"""
import json
import os
import re

import numpy as np
import pytest

from tensormol_gb300 import params as P

HERE = os.path.dirname(os.path.abspath(__file__))
API_CU = os.path.join(os.path.dirname(HERE), "tensormol_gb300", "csrc", "tm_api.cu")

# PARAMS defaults that differ from TMParams.py on purpose, with the
# reference's own value and the reason
INTENTIONAL = {
    "HiddenLayers": ([200, 200, 200], "the benchmarked networks are 3 x 512 wide"),
    "KeepProb": (0.7, "a training setting; evaluation runs with keep = 1 "
                      "(TFBehlerParinelloSymEE.py:1448)"),
    "EECutoffOn": (4.4, "the DSF/elu model raises unless it is 0 "
                        "(TFBehlerParinelloSymEE.py:725-726); the samples set 0"),
    "MDLogTrajectory": (True, "a library call writes no files unless asked"),
}


@pytest.fixture(scope="module")
def g(golden_loader):
    return golden_loader("constants")


def test_units(g):
    assert P.BOHRPERA == float(g["BOHRPERA"])
    assert P.KJPERHARTREE == float(g["KJPERHARTREE"])
    assert P.JOULEPERHARTREE == float(g["JOULEPERHARTREE"])
    assert P.IDEALGASR == float(g["IDEALGASR"])


def test_element_tables(g):
    for z in range(1, 11):
        assert P.ATOMICMASSES[z] == g["ATOMICMASSES"][z - 1], z
        assert P.C6_COFF[z] == g["C6_coff"][z - 1], z
        assert P.ATOMIC_VDW_RADIUS[z] == g["atomic_vdw_radius"][z - 1], z


def _cu_array(src, name):
    m = re.search(r"static const double %s\[\d+\] = \{([^}]*)\};" % name, src)
    return np.array([float(v) for v in m.group(1).split(",")])


def test_library_host_tables(g):
    """tm_api.cu's own copies: bohr per angstrom, J per Hartree, C6 and vdW
    radius tables indexed by atomic number."""
    src = open(API_CU).read()
    bohr = float(re.search(r"static const double kBohr = ([0-9.eE+-]+);", src).group(1))
    kj, scale = re.search(r"static const double kJph = ([0-9.eE+-]+) \* ([0-9.eE+-]+);", src).groups()
    assert bohr == float(g["BOHRPERA"])
    assert float(kj) * float(scale) == float(g["JOULEPERHARTREE"])
    np.testing.assert_array_equal(_cu_array(src, "kC6")[1:], g["C6_coff"])
    np.testing.assert_array_equal(_cu_array(src, "kR0")[1:], g["atomic_vdw_radius"])


def test_params_defaults(g):
    ref = json.loads(str(g["tmparams"]))
    checked = 0
    for key, ours in P.PARAMS.items():
        if key not in ref:
            continue   # e.g. MNHChain, which the reference reads without defining
        theirs = ref[key]
        if key in INTENTIONAL:
            assert theirs == INTENTIONAL[key][0], key
            continue
        if isinstance(ours, (list, tuple)):
            assert list(ours) == list(theirs), key
        else:
            assert ours == theirs, key
        checked += 1
    assert checked >= 30


def test_dsf_kernel_and_elu_constants(g):
    r, rc, alpha = g["dsf_r"], float(g["dsf_rc"]), float(g["dsf_alpha"])
    # math.erfc here, scipy.special.erfc in the reference: they differ in the
    # last bits, which the cancellation near the cutoff (values ~1e-7) shows
    np.testing.assert_allclose([P.dsf(x, rc, alpha) for x in r], g["dsf"], rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose([P.dsf_gradient(x, rc, alpha) for x in r], g["dsf_grad"],
                               rtol=1e-13, atol=1e-16)
    c = P.coulomb_constants()
    assert c["r_lr"] == rc and c["alpha"] == alpha
    np.testing.assert_allclose(c["elu_shift"], float(g["elu_shift"]), rtol=1e-14)
    np.testing.assert_allclose(c["elu_a"], float(g["elu_alpha"]), rtol=1e-14)
