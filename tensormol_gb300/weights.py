"""Trained TensorMol BP+EE weights in this package's layout.

The reference's networks are TensorFlow variables named by element and layer
(TFNetworks/TFBehlerParinelloSymEE.py:915-995):

    EnergyNet/{Z}_hidden{k}/weights            [fan_in, fan_out]
    EnergyNet/{Z}_hidden{k}/biaseslayer{k-1}   [fan_out]
    EnergyNet/{Z}_regression_linear/weights    [hidden[-1], 1]
    EnergyNet/{Z}_regression_linear/biases     [1]
    DipoleNet/{Z}_hidden{k}_charge/weights, .../biases
    DipoleNet/{Z}_regression_linear_charge/weights, .../biases

``load_tensormol_weights`` maps any name -> array mapping holding those names
(an ``.npz`` file, or the dict that ``checkpoint_to_npz`` writes) to the
``{"E": {Z: [(W, b), ...]}, "Q": {...}}`` structure ``BPEEModel`` takes.
``checkpoint_to_npz`` reads a TensorFlow checkpoint and needs TensorFlow, which
is not part of this package; run it wherever TensorFlow is installed.
"""
from __future__ import annotations

import numpy as np


def _get(src, name):
    for key in (name, name + ":0"):
        if key in src:
            return np.asarray(src[key], dtype=np.float64)
    raise KeyError(f"missing weight tensor {name!r}")


def load_tensormol_weights(src, eles, n_hidden):
    """src: mapping (or path to an .npz) of TensorMol variable names to arrays;
    eles: atomic numbers of the model; n_hidden: number of hidden layers."""
    if isinstance(src, str):
        src = dict(np.load(src))
    out = {"E": {}, "Q": {}}
    for e in eles:
        layers_e, layers_q = [], []
        for k in range(1, n_hidden + 1):
            layers_e.append((_get(src, f"EnergyNet/{e}_hidden{k}/weights"),
                             _get(src, f"EnergyNet/{e}_hidden{k}/biaseslayer{k - 1}")))
            layers_q.append((_get(src, f"DipoleNet/{e}_hidden{k}_charge/weights"),
                             _get(src, f"DipoleNet/{e}_hidden{k}_charge/biases")))
        layers_e.append((_get(src, f"EnergyNet/{e}_regression_linear/weights"),
                         _get(src, f"EnergyNet/{e}_regression_linear/biases")))
        layers_q.append((_get(src, f"DipoleNet/{e}_regression_linear_charge/weights"),
                         _get(src, f"DipoleNet/{e}_regression_linear_charge/biases")))
        for layers in (layers_e, layers_q):
            for (W, b), nxt in zip(layers, layers[1:] + [None]):
                if W.ndim != 2 or b.shape != (W.shape[1],):
                    raise ValueError(f"element {e}: weight {W.shape} does not match bias {b.shape}")
                if nxt is not None and nxt[0].shape[0] != W.shape[1]:
                    raise ValueError(f"element {e}: layer widths do not chain")
        out["E"][e] = layers_e
        out["Q"][e] = layers_q
    return out


def tensormol_names(weights):
    """The inverse mapping: this package's weights under the reference's
    variable names (for round trips and for writing fixtures)."""
    out = {}
    for e, layers in weights["E"].items():
        for k, (W, b) in enumerate(layers[:-1], start=1):
            out[f"EnergyNet/{e}_hidden{k}/weights"] = W
            out[f"EnergyNet/{e}_hidden{k}/biaseslayer{k - 1}"] = b
        out[f"EnergyNet/{e}_regression_linear/weights"] = layers[-1][0]
        out[f"EnergyNet/{e}_regression_linear/biases"] = layers[-1][1]
    for e, layers in weights["Q"].items():
        for k, (W, b) in enumerate(layers[:-1], start=1):
            out[f"DipoleNet/{e}_hidden{k}_charge/weights"] = W
            out[f"DipoleNet/{e}_hidden{k}_charge/biases"] = b
        out[f"DipoleNet/{e}_regression_linear_charge/weights"] = layers[-1][0]
        out[f"DipoleNet/{e}_regression_linear_charge/biases"] = layers[-1][1]
    return out


def checkpoint_to_npz(checkpoint_prefix, out_path):
    """Copy every variable of a TensorFlow checkpoint (the reference's
    ``networks/<name>/<name>-chk-*`` files) into an .npz keyed by name."""
    try:
        import tensorflow as tf   # noqa: F401  (not a dependency of this package)
    except ImportError as exc:
        raise RuntimeError("checkpoint_to_npz needs TensorFlow; run it where TensorFlow is "
                           "installed and copy the .npz") from exc
    reader = tf.train.load_checkpoint(checkpoint_prefix)
    arrays = {name: reader.get_tensor(name) for name in reader.get_variable_to_shape_map()}
    np.savez(out_path, **arrays)
    return sorted(arrays)
