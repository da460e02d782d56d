"""Network shapes, activations and trained-weight loading on the device,
against the FP64 oracle (FP32 path: 1e-5 eV/atom, 1e-4 eV/A max-abs).

* hidden widths other than 3 x 512, including the reference's own default
  HiddenLayers = [200]*3 (TMParams.py:66), two- and one-layer networks and
  unequal widths (the layer kernel pads every width to a multiple of 256);
* every activation of Instance.AssignActivation (TFNetworks/TFInstance.py:
  108-140);
* weights stored under the reference's TensorFlow variable names
  (TFBehlerParinelloSymEE.py:915-995), written to an .npz and read back by
  tensormol_gb300.weights, evaluated on the device.

Biases are non-zero here (random-init networks have zero biases), as in
trained networks.
"""
import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import EV_PER_HARTREE, JOULEPERHARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu

E_TOL = 1e-5
F_TOL = 1e-4


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import model
    return model


def _weights(eles, hidden, seed=5):
    W = systems.random_weights(eles, descriptor_width(len(eles)), hidden=hidden, seed=seed)
    rng = np.random.default_rng(seed + 100)
    for net in W:
        for e in W[net]:
            W[net][e] = [(Wm, rng.normal(scale=0.05, size=b.shape)) for (Wm, b) in W[net][e]]
    return W


def _check(gpu, b, eles, W, act, hidden):
    p = dict(PARAMS)
    p["NeuronType"] = act
    p["HiddenLayers"] = list(hidden)
    m = gpu.BPEEModel(eles, W, params=p, precision="fp32")
    s = m.system(b.x, b.Z, b.offsets)
    out = s.energy_force(b.x, True)
    ref = orc.OpenSystemOracle(orc.Model(eles, W, p), b.x, b.Z, b.offsets).terms(b.x)
    n_per = np.diff(b.offsets)
    dE = np.max(np.abs(out["Etotal"] - ref["Etotal"]) * EV_PER_HARTREE / n_per)
    dF = np.abs(out["force"] - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    s.close()
    m.close()
    assert dE < E_TOL and dF < F_TOL, (act, hidden, dE, dF)


@pytest.mark.parametrize("hidden", [(200, 200, 200), (256, 128), (512,), (300, 700, 100)])
@pytest.mark.parametrize("act", ["sigmoid_with_param", "relu"])
def test_hidden_layer_shapes(gpu, hidden, act):
    w = systems.water_cluster_60(seed=0)
    _check(gpu, w, [1, 8], _weights([1, 8], hidden), act, hidden)


def test_reference_default_network_on_chno(gpu):
    """The reference's default network (3 x 200, relu) on a CHNO batch."""
    b = systems.chno_batch(nmol=24, seed=3)
    hidden = (200, 200, 200)
    _check(gpu, b, [1, 6, 7, 8], _weights([1, 6, 7, 8], hidden), "relu", hidden)


@pytest.mark.parametrize("act", ["tanh", "softplus", "elu"])
def test_activations(gpu, act):
    w = systems.water_cluster_60(seed=0)
    _check(gpu, w, [1, 8], _weights([1, 8], (512, 512, 512)), act, (512, 512, 512))


def test_weights_by_reference_names_on_device(gpu, tmp_path):
    from tensormol_gb300.weights import load_tensormol_weights, tensormol_names
    hidden = (200, 200, 200)
    W = _weights([1, 8], hidden, seed=9)
    path = str(tmp_path / "water_net.npz")
    np.savez(path, **tensormol_names(W))
    loaded = load_tensormol_weights(path, [1, 8], len(hidden))
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    p["HiddenLayers"] = list(hidden)
    w = systems.water_cluster_60(seed=0)
    m = gpu.BPEEModel([1, 8], loaded, params=p, precision="fp32")
    s = m.system(w.x, w.Z, w.offsets)
    out = s.energy_force(w.x, True)
    ref = orc.OpenSystemOracle(orc.Model([1, 8], W, p), w.x, w.Z, w.offsets).terms(w.x)
    dE = abs(out["Etotal"][0] - ref["Etotal"][0]) * EV_PER_HARTREE / w.natoms
    dF = np.abs(out["force"] - ref["force"]).max() / JOULEPERHARTREE * EV_PER_HARTREE
    assert dE < E_TOL and dF < F_TOL, (dE, dF)
