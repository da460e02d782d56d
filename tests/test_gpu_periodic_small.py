"""Periodic cells smaller than twice the largest cutoff (the reference then
tessellates more than one shell of images, Periodic.py:143-147): 64 H2O in a
12.4 A cell with the default 15 A Coulomb cutoff, cubic and sheared, against
the oracle's two-shell (125-image) tessellation. The library evaluates such a
cell as the smallest supercell whose plane spacings reach twice the cutoff
(27 copies here) and hands back copy 0's forces and the energy per cell:
FP32 energies within 1e-5 eV/atom, forces within 1e-4 eV/A. Lists, the
images-fixed force and MD of such a cell are refused with TM_E_UNSUPPORTED.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu

A = 3.1 * 4   # 4 x 4 x 4 lattice sites of 3.1 A


@pytest.fixture(scope="module")
def small():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import md, model
    b = systems.water(64, seed=8, spacing=3.1, box=A, n_side=4)
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    return model, md, b, p, W


@pytest.mark.parametrize("shear", [0.0, 0.2])
def test_small_cell_energy_force(small, shear):
    model, md, b, p, W = small
    B = np.array([[A, 0.0, 0.0], [shear * A, A, 0.0], [0.0, -0.5 * shear * A, A]])
    x = orc.modulo_lattice((b.x / A) @ B, B)
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    s = m.system(x, b.Z, None, B)
    out = s.energy_force(x, True, charges=True)
    ref = orc.PeriodicOracle(orc.Model([1, 8], W, p), x, b.Z, B, ntess=2).terms(x)
    dE = abs(out["Etotal"][0] - ref["Etotal"][0]) * EV_PER_HARTREE / len(b.Z)
    dF = np.abs(out["force"] - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    dq = np.abs(out["charge"] - ref["charge"]).max()
    print(f"cell {A:.1f} A shear {shear}: dE/atom={dE:.2e} eV  max|dF|={dF:.2e} eV/A  max|dq|={dq:.1e}")
    assert dE < 1e-5 and dF < 1e-4 and dq < 2e-6, (dE, dF, dq)
    assert out["force"].shape == (len(b.Z), 3) and s.positions().shape == (len(b.Z), 3)


def test_small_cell_refuses_what_it_cannot_reproduce(small):
    from tensormol_gb300 import _lib
    model, md, b, p, W = small
    B = np.eye(3) * A
    x = orc.modulo_lattice(b.x, B)
    m = model.BPEEModel([1, 8], W, params=p, precision="fp32")
    s = m.system(x, b.Z, None, B)
    s.energy_force(x, True)
    code = _lib.ERROR_CODES["TM_E_UNSUPPORTED"]
    for call in (lambda: s.export_nlist(),
                 lambda: s.energy_force(x, True, reference_periodic_force=True),
                 lambda: md.DeviceMD(s, "nve")):
        with pytest.raises(_lib.TmError) as err:
            call()
        assert err.value.code == code
