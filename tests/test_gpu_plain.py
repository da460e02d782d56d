"""The plain-autograd comparator (tensormol_gb300/plain.py) against the FP64
oracle: the reference's graph structure as framework ops on the GPU over the
library's exported lists, forces by torch.autograd.grad. Energies within
1e-5 eV/atom and forces within 1e-4 eV/A max-abs for water (smooth
activation). For CHNO molecules the bound is 3e-4 eV/A: the reference's
angle form takes acos of an FP32 cosine clamped to +-(1 - 1e-7), whose
derivative 1/sin(theta) magnifies FP32 rounding in nearly collinear triples
(measured 1.5e-4 eV/A; the fused path forms sin(theta) from a cross product
instead and stays within 1e-4)."""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import model, plain
    return torch, model, plain


@pytest.mark.parametrize("case", ["water60", "chno8"])
def test_plain_autograd_against_oracle(gpu, case):
    torch, model, plain = gpu
    if case == "water60":
        b, eles = systems.water_cluster_60(seed=0), [1, 8]
    else:
        b, eles = systems.chno_batch(nmol=8, seed=3), [1, 6, 7, 8]
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights(eles, descriptor_width(len(eles)), seed=7)
    m = model.BPEEModel(eles, W, params=p, precision="fp32")
    s = m.system(b.x, b.Z, b.offsets)
    s.build_nlist()
    pl = plain.PlainAutograd(m, W)
    pl.prepare(s)
    E, F = pl.energy_force(torch.tensor(b.x, dtype=torch.float64, device="cuda"))
    E, F = E.cpu().numpy(), F.cpu().numpy()
    ref = orc.OpenSystemOracle(orc.Model(eles, W, p), b.x, b.Z, b.offsets).terms(b.x)
    n_per = np.diff(b.offsets)
    dE = np.max(np.abs(E - ref["Etotal"]) * EV_PER_HARTREE / n_per)
    dF = np.abs(F - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    f_tol = 1e-4 if case == "water60" else 3e-4
    assert dE < 1e-5 and dF < f_tol, (dE, dF)
