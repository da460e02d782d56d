"""Parameters and physical constants of the BP+EE energy-and-force path.

The keys of ``PARAMS`` carry the same names and defaults as the reference's
global parameter dictionary (``TensorMol/TMParams.py:8-171``) for every key the
energy/force path and the integrators read, so that scripts which mutate
``PARAMS[...]`` before building a model keep working unchanged.

Two defaults of the reference are unusable on this path and are set the way
every working script of the reference sets them:

* ``EECutoffOn`` must be 0 for the DSF/elu instance, which raises otherwise
  (``TFNetworks/TFBehlerParinelloSymEE.py:724-725``); the reference default is 4.4.
* ``KeepProb`` must be a list (its length sets the layer count,
  ``TFBehlerParinelloSymEE.py:735``); at evaluation every entry is 1.0
  (``TFBehlerParinelloSymEE.py:1448``).

The physical constants restate ``TensorMol/PhysicalData.py`` values used here.
"""
from __future__ import annotations

import math

import numpy as np

# ---------------------------------------------------------------------------
# Physical data (TensorMol/PhysicalData.py:22-57)
# ---------------------------------------------------------------------------
BOHRPERA = 1.889725989                      # PhysicalData.py:30
KJPERHARTREE = 2625.499638                  # PhysicalData.py:36
JOULEPERHARTREE = KJPERHARTREE * 1000.0     # PhysicalData.py:37
IDEALGASR = 8.3144621                       # PhysicalData.py:50, J/(mol K)
EV_PER_HARTREE = 27.211386245988            # CODATA 2018; used only in tolerances

# Atomic masses in amu for Z = 1..10 (PhysicalData.py:21), converted to kg/mol
# exactly as the reference does (PhysicalData.py:57: 0.000999977 * amu).
_AMU = [1.00794, 4.002602, 6.941, 9.012182, 10.811, 12.0107, 14.0067,
        15.9994, 18.9984032, 20.1791]
ATOMICMASSES = {z + 1: 0.000999977 * m for z, m in enumerate(_AMU)}

# Grimme C6 coefficients (J nm^6 / mol) and vdW radii (Angstrom),
# PhysicalData.py:25-26.
C6_COFF = {1: 0.14, 2: 0.08, 3: 1.16, 4: 1.61, 5: 3.13, 6: 1.75, 7: 1.23,
           8: 0.70, 9: 0.75, 10: 0.63}
ATOMIC_VDW_RADIUS = {1: 1.001, 2: 1.012, 3: 0.825, 4: 1.408, 5: 1.485,
                     6: 1.452, 7: 1.397, 8: 1.342, 9: 1.287, 10: 1.243}

# ---------------------------------------------------------------------------
# PARAMS (TMParams.py)
# ---------------------------------------------------------------------------
PARAMS = {
    # ANI-1 symmetry functions (TMParams.py:26-37)
    "AN1_r_Rc": 4.6,
    "AN1_a_Rc": 3.1,
    "AN1_eta": 4.0,
    "AN1_zeta": 8.0,
    "AN1_num_r_Rs": 32,
    "AN1_num_a_Rs": 8,
    "AN1_num_a_As": 8,
    # network (TMParams.py:57,66,74,79)
    "NeuronType": "relu",
    "HiddenLayers": [512, 512, 512],
    "KeepProb": [1.0, 1.0, 1.0, 1.0],
    "sigmoid_alpha": 100.0,
    # electrostatic embedding (TMParams.py:140-154)
    "AddEcc": True,
    "Poly_Width": 4.6,
    "Elu_Width": 4.6,
    "EECutoffOn": 0.0,
    "EECutoffOff": 15.0,
    "DSFAlpha": 0.18,
    # MD (TMParams.py:115-127)
    "MDMaxStep": 20000,
    "MDdt": 0.2,
    "MDTemp": 300.0,
    "MDV0": "Random",
    "MDThermostat": None,
    "MDLogTrajectory": False,
    # Nose-Hoover chain length; the reference reads this key without
    # defining it (Simulations/SimpleMD.py:220).
    "MNHChain": 3,
    # geometry optimisation (TMParams.py:96-114)
    "OptMaxCycles": 50,
    "OptThresh": 0.0001,
    "OptMaxStep": 0.1,
    "OptStepSize": 0.1,
    "OptMomentum": 0.5,
    "OptMomentumDecay": 0.8,
    "GSSearchAlpha": 0.05,
    "SDStep": 0.05,
    "NebSolver": "Verlet",
    "NebNumBeads": 18,
    "NebK": 0.07,
    "NebClimbingImage": True,
    "RemoveInvariant": True,
}

ACTIVATIONS = {"relu": 0, "sigmoid_with_param": 1, "softplus": 2, "tanh": 3,
               "elu": 4}


def ani1_grids(params=None):
    """Shift grids of the ANI-1 functions, ``SetANI1Param``
    (TFNetworks/TFBehlerParinelloSymEE.py:738-777; TMParams.py:35-37).

    Returns (radial Rs [nr], angular Rs [na_rs], angular theta_s [na_as]).
    """
    p = PARAMS if params is None else params
    nr, nars, naas = p["AN1_num_r_Rs"], p["AN1_num_a_Rs"], p["AN1_num_a_As"]
    rs_r = np.array([p["AN1_r_Rc"] * i / nr for i in range(nr)], dtype=np.float64)
    rs_a = np.array([p["AN1_a_Rc"] * i / nars for i in range(nars)], dtype=np.float64)
    th = np.array([2.0 * math.pi * i / naas for i in range(naas)], dtype=np.float64)
    return rs_r, rs_a, th


def element_pairs(eles):
    """i <= j element pairs in order (TFBehlerParinelloSymEE.py:678-682)."""
    return [(eles[i], eles[j]) for i in range(len(eles)) for j in range(i, len(eles))]


def descriptor_width(n_ele, params=None):
    """nele*nr + nelep*na_rs*na_as (TFBehlerParinelloSymEE.py:772)."""
    p = PARAMS if params is None else params
    nelep = n_ele * (n_ele + 1) // 2
    return n_ele * p["AN1_num_r_Rs"] + nelep * p["AN1_num_a_Rs"] * p["AN1_num_a_As"]


def dsf(r, rc, alpha):
    """Damped shifted force kernel value (Util.py:172-181)."""
    from math import erfc, exp
    if r > rc:
        return 0.0
    xx = alpha * rc
    zz = erfc(xx) / rc
    yy = 1.1283791671 * alpha * exp(-xx * xx) / rc
    return erfc(alpha * r) / r - zz + (r - rc) * (zz / rc + yy)


def dsf_gradient(r, rc, alpha):
    """Derivative of the DSF kernel (Util.py:183-192)."""
    from math import erfc, exp
    if r > rc:
        return 0.0
    xx = alpha * rc
    zz = erfc(xx) / rc
    yy = 1.1283791671 * alpha * exp(-xx * xx) / rc
    return -((erfc(alpha * r) / r / r + 1.1283791671 * alpha * exp(-alpha * r * alpha * r) / r)
             - (zz / rc + yy))


def coulomb_constants(params=None):
    """Constants of ``TFCoulombEluSRDSFLR`` in atomic units.

    alpha = DSFAlpha / BOHRPERA (RawSymFunc.py:1323); R_lr = EECutoffOff * BOHRPERA
    (RawSymFunc.py:1324); the short-range elu piece starts at Elu_Width * BOHRPERA
    (TFBehlerParinelloSymEE.py:1012) with shift/slope from DSF/DSF_Gradient at that
    radius (TFBehlerParinelloSymEE.py:727-729).
    """
    p = PARAMS if params is None else params
    alpha = p["DSFAlpha"] / BOHRPERA
    r_lr = p["EECutoffOff"] * BOHRPERA
    r_sr = p["Elu_Width"] * BOHRPERA
    shift = dsf(r_sr, r_lr, alpha)
    slope = dsf_gradient(r_sr, r_lr, alpha)
    return dict(alpha=alpha, r_lr=r_lr, r_sr=r_sr, elu_shift=shift, elu_a=slope)


def vdw_tables(eles, params=None):
    """Per-element C6 (atomic units) and vdW radius (bohr),
    TFBehlerParinelloSymEE.py:719-723."""
    c6 = np.array([C6_COFF[e] * (BOHRPERA * 10.0) ** 6.0 / JOULEPERHARTREE for e in eles])
    r0 = np.array([ATOMIC_VDW_RADIUS[e] * BOHRPERA for e in eles])
    return c6, r0
