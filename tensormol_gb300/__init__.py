"""GB300-native (sm_103a) implementation of TensorMol's BP+EE energy-and-force path.

Public surface:
  params      PARAMS and physical constants (names of TensorMol/TMParams.py)
  systems     seeded synthetic systems and random-init weights
  model       BPEEModel / System / TFMolManage / EnergyAndForce (the drop-in)
  md          VelocityVerlet and Nose / Nose-Hoover-chain integrators on the device
  plain       the plain-autograd comparison path (torch ops over the same lists)
The compute path is libtmgpu.so (include/tmgpu.h); there is no CPU fallback.
"""
from .params import PARAMS  # noqa: F401
