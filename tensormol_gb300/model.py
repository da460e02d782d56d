"""Host-side mirror of TensorMol's BP+EE evaluation interface, backed by libtmgpu.

``BPEEModel`` plays the part of ``MolInstance_DirectBP_EE_SymFunction``
(TFNetworks/TFBehlerParinelloSymEE.py:656-1501) and ``TFMolManage`` the part of
the manager's evaluation methods (TFNetworks/TFMolManage.py:1260-1439): same
method names, argument meaning, return tuples and units, so existing
``EnAndForce`` closures, optimisers, MD and NEB drivers can call it unchanged.
All arithmetic runs in the CUDA library; this module only moves arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import JOULEPERHARTREE, PARAMS, ACTIVATIONS, descriptor_width, element_pairs

_F64 = np.float64
# element symbols by atomic number (PhysicalData.py:17-18), Z = 1..10 here
_SYMBOLS = ["X", "H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"]


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


class Context:
    """One CUDA stream + status word + HBM budget on one device (tm_ctx)."""

    def __init__(self, device=0, hbm_budget_bytes=0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(None, self.lib.tm_ctx_create(device, hbm_budget_bytes, ctypes.byref(h)))
        self.h = h

    def check(self, rc):
        _lib.check(self.h, rc)

    @property
    def launches(self):
        return int(self.lib.tm_ctx_launch_count(self.h))

    @property
    def bytes_in_use(self):
        return int(self.lib.tm_ctx_bytes_in_use(self.h))

    @property
    def stream(self):
        return self.lib.tm_ctx_stream(self.h)

    def set_stream(self, stream_ptr):
        self.check(self.lib.tm_ctx_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def close(self):
        if self.h:
            self.lib.tm_ctx_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass


_DEFAULT_CTX = None


def default_context():
    global _DEFAULT_CTX
    if _DEFAULT_CTX is None:
        _DEFAULT_CTX = Context(0)
    return _DEFAULT_CTX


class BPEEModel:
    """Per-element energy and charge networks on ANI-1 descriptors.

    eles: sorted atomic numbers. weights: {"E": {ele: [(W, b), ...]}, "Q": {...}}
    with W[fan_in, fan_out] per layer (the reference's tf.matmul orientation) and
    a final [hidden, 1] regression layer. params: a PARAMS-like dict
    (tensormol_gb300.params.PARAMS keys). precision: "fp32" (3-pass split TF32
    tensor cores, FP32-level error) or "bf16" (one BF16 pass).
    """

    def __init__(self, eles, weights, params=None, precision="fp32", has_vdw=True, ctx=None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.p = dict(PARAMS if params is None else params)
        self.eles = [int(e) for e in eles]
        self.eles_pairs = element_pairs(self.eles)
        self.precision = precision
        self.has_vdw = bool(has_vdw)
        hidden = list(self.p["HiddenLayers"])
        d = _lib.tm_model_desc()
        d.n_elements = len(self.eles)
        for i, e in enumerate(self.eles):
            d.elements[i] = e
        d.n_hidden = len(hidden)
        for i, h in enumerate(hidden):
            d.hidden[i] = int(h)
        d.activation = ACTIVATIONS[self.p["NeuronType"]]
        d.sigmoid_alpha = float(self.p["sigmoid_alpha"])
        d.r_rc, d.a_rc = float(self.p["AN1_r_Rc"]), float(self.p["AN1_a_Rc"])
        d.eta, d.zeta = float(self.p["AN1_eta"]), float(self.p["AN1_zeta"])
        d.n_r_rs, d.n_a_rs, d.n_a_as = (int(self.p["AN1_num_r_Rs"]), int(self.p["AN1_num_a_Rs"]),
                                        int(self.p["AN1_num_a_As"]))
        d.ee_cut_on, d.ee_cut_off = float(self.p["EECutoffOn"]), float(self.p["EECutoffOff"])
        d.elu_width, d.dsf_alpha = float(self.p["Elu_Width"]), float(self.p["DSFAlpha"])
        d.poly_width = float(self.p["Poly_Width"])
        d.add_ecc = 1 if self.p["AddEcc"] else 0
        d.has_vdw = 1 if has_vdw else 0
        d.precision = _lib.TM_PREC[precision]
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.tm_model_create(self.ctx.h, ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        self.D = int(self.lib.tm_model_descriptor_width(h))
        assert self.D == descriptor_width(len(self.eles), self.p)
        for net_i, net in enumerate(("E", "Q")):
            for e_i, e in enumerate(self.eles):
                for l_i, (W, b) in enumerate(weights[net][e]):
                    W = np.ascontiguousarray(W, dtype=_F64)
                    b = np.ascontiguousarray(b, dtype=_F64).reshape(-1)
                    self.ctx.check(self.lib.tm_model_set_layer(h, net_i, e_i, l_i, _ptr(W), _ptr(b),
                                                               W.shape[0], W.shape[1]))
        self.ctx.check(self.lib.tm_model_finalize(h))

    def system(self, x, Z, offsets=None, cell=None):
        return System(self, x, Z, offsets, cell)

    def close(self):
        if self.h:
            self.lib.tm_model_destroy(self.h)
            self.h = None


class System:
    """Device-resident atoms of a batch of molecules (tm_system)."""

    def __init__(self, model, x, Z, offsets=None, cell=None):
        self.model = model
        self.ctx = model.ctx
        self.lib = model.lib
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        self.N = int(Z.shape[0])
        if offsets is None:
            offsets = np.array([0, self.N], dtype=np.int64)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        self.nmol = int(self.offsets.shape[0] - 1)
        self.Z = Z
        self.cell = None if cell is None else np.ascontiguousarray(cell, dtype=_F64).reshape(3, 3)
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.tm_system_create(model.h, self.N, self.nmol, _ptr(Z), _ptr(self.offsets),
                                                 _ptr(self.cell), ctypes.byref(h)))
        self.h = h
        if x is not None:
            self.set_positions(x)

    # -- positions and lists ------------------------------------------------
    def set_positions(self, x):
        x = np.ascontiguousarray(x, dtype=_F64)
        assert x.shape == (self.N, 3)
        self.ctx.check(self.lib.tm_system_set_positions(self.h, _ptr(x), 0))

    def positions(self):
        x = np.empty((self.N, 3))
        self.ctx.check(self.lib.tm_system_get_positions(self.h, _ptr(x), 0))
        return x

    def build_nlist(self):
        self.ctx.check(self.lib.tm_system_build_nlist(self.h))

    def nlist_counts(self):
        c = np.zeros(4, dtype=np.int64)
        self.ctx.check(self.lib.tm_system_nlist_counts(self.h, _ptr(c)))
        return dict(pairs=int(c[0]), triples=int(c[1]), ee_pairs=int(c[2]), max_radial=int(c[3]))

    def export_nlist(self):
        """(RadpEle [P,4], AngtEle [T,5], mil_j [P,4], mil_jk [T,4]) as the
        reference's NeighborListSet returns them (molecule-local indices)."""
        c = self.nlist_counts()
        P, T = c["pairs"], c["triples"]
        radp = np.zeros((P, 4), np.int64)
        angt = np.zeros((T, 5), np.int64)
        milj = np.zeros((P, 4), np.int64)
        miljk = np.zeros((T, 4), np.int64)
        self.ctx.check(self.lib.tm_system_export_nlist(self.h, _ptr(radp), _ptr(angt), _ptr(milj),
                                                       _ptr(miljk), 0))
        return radp, angt, milj, miljk

    def descriptors(self):
        """FP32 descriptor rows [N, D] in atom order (diagnostic)."""
        G = np.zeros((self.N, self.model.D), dtype=np.float32)
        self.ctx.check(self.lib.tm_system_descriptors(self.h, _ptr(G)))
        return G

    def layer_outputs(self, layer):
        """[2, N, width] outputs of hidden layer ``layer`` of both networks
        from the last evaluation (call after ``energy_force(x, False)``): the
        activations, or for the last hidden layer w_out * act'(z)."""
        width = int(self.model.p["HiddenLayers"][layer])
        out = np.zeros((2, self.N, width), dtype=np.float32)
        self.ctx.check(self.lib.tm_system_layer_outputs(self.h, int(layer), _ptr(out)))
        return out

    def refined_units(self):
        """Hidden units the last evaluation recomputed in FP64 near the relu
        kink (FP32 mode with relu; 0 otherwise)."""
        n = ctypes.c_int64()
        self.ctx.check(self.lib.tm_system_refined_units(self.h, ctypes.byref(n)))
        return int(n.value)

    def export_ee(self):
        n = self.nlist_counts()["ee_pairs"]
        out = np.zeros((max(n, 1), 3), np.int64)
        self.ctx.check(self.lib.tm_system_export_ee(self.h, _ptr(out), n, 0))
        return out[:n]

    # -- evaluation ----------------------------------------------------------
    def energy_force(self, x=None, do_force=True, charges=False, reference_periodic_force=False):
        flags = 0 if do_force else _lib.TM_F_ENERGY_ONLY
        if reference_periodic_force:
            flags |= _lib.TM_F_REFERENCE_PERIODIC_FORCE
        xa = None if x is None else np.ascontiguousarray(x, dtype=_F64)
        E = np.zeros((self.nmol, 4))
        F = np.zeros((self.N, 3)) if do_force else None
        q = np.zeros(self.N) if charges else None
        dip = np.zeros((self.nmol, 3)) if charges else None
        Ea = np.zeros(self.N) if charges else None
        self.ctx.check(self.lib.tm_energy_force(self.h, _ptr(xa), flags, _ptr(E), _ptr(F), _ptr(q),
                                                _ptr(dip), _ptr(Ea)))
        out = dict(Etotal=E[:, 0].copy(), Ebp=E[:, 1].copy(), Ecc=E[:, 2].copy(), Evdw=E[:, 3].copy())
        if do_force:
            out["force"] = F
        if charges:
            out.update(charge=q, dipole=dip, Ebp_atom=Ea)
        return out

    def energy_force_device(self, x_dev_ptr, E_dev_ptr, F_dev_ptr, flags=0):
        """Device-pointer variant (TM_F_DEVICE_IO): x, E[nmol,4], F[N,3] live in
        HBM (e.g. torch tensors' data_ptr()) on the context's stream."""
        self.ctx.check(self.lib.tm_energy_force(self.h, ctypes.c_void_p(x_dev_ptr),
                                                flags | _lib.TM_F_DEVICE_IO,
                                                ctypes.c_void_p(E_dev_ptr), ctypes.c_void_p(F_dev_ptr),
                                                None, None, None))

    def close(self):
        if self.h:
            self.lib.tm_system_destroy(self.h)
            self.h = None


def _padded(mols):
    nmol = len(mols)
    maxn = max(len(m.atoms) for m in mols)
    return nmol, maxn


class TFMolManage:
    """Evaluation half of the reference's manager (TFMolManage.py:1260-1439).

    ``Instances`` is the BPEEModel. Systems are cached per (Z, offsets, cell)
    signature, the way the reference rebuilds its graph only on a shape change
    (TFBehlerParinelloSymEE.py:1436-1441).
    """

    def __init__(self, model):
        self.Instances = model
        self._cache = {}

    def _system(self, Z, offsets, cell=None):
        key = (Z.tobytes(), offsets.tobytes(), None if cell is None else cell.tobytes())
        s = self._cache.get(key)
        if s is None:
            if len(self._cache) > 16:
                for v in self._cache.values():
                    v.close()
                self._cache.clear()
            s = System(self.Instances, None, Z, offsets, cell)
            self._cache[key] = s
        return s

    def _check_cuts(self, Rr_cut, Ra_cut, Ree_cut):
        p = self.Instances.p
        if (abs(Rr_cut - p["AN1_r_Rc"]) > 1e-12 or abs(Ra_cut - p["AN1_a_Rc"]) > 1e-12
                or abs(Ree_cut - p["EECutoffOff"]) > 1e-12):
            raise Exception("cutoffs must match the model's PARAMS (AN1_r_Rc, AN1_a_Rc, EECutoffOff)")

    def EvalBPDirectEELinearSingle(self, mol, Rr_cut, Ra_cut, Ree_cut, HasVdw=False):
        """Returns (Etotal, Ebp, Ebp_atom, Ecc, Evdw, dipole, charge, force) with
        HasVdw, else (Etotal, Ebp, Ecc, dipole, charge, force); force in J/mol/A
        with shape [1, N, 3] (TFMolManage.py:1410-1439)."""
        self._check_cuts(Rr_cut, Ra_cut, Ree_cut)
        if bool(HasVdw) != self.Instances.has_vdw:
            raise Exception("HasVdw must match the model")
        Z = np.ascontiguousarray(mol.atoms, dtype=np.int32)
        x = np.ascontiguousarray(mol.coords, dtype=_F64)
        x = np.where(np.isfinite(x), x, np.nan)
        if not np.all(np.isfinite(x)):
            raise Exception("Please check your inputs")
        s = self._system(Z, np.array([0, len(Z)], dtype=np.int64))
        o = s.energy_force(x, True, charges=True)
        N = len(Z)
        force = o["force"].reshape(1, N, 3)
        if HasVdw:
            return (o["Etotal"], o["Ebp"], o["Ebp_atom"].reshape(1, N), o["Ecc"], o["Evdw"],
                    o["dipole"], o["charge"].reshape(1, N), force)
        return o["Etotal"], o["Ebp"], o["Ecc"], o["dipole"], o["charge"].reshape(1, N), force

    EvalBPDirectEEUpdateSingle = EvalBPDirectEELinearSingle

    def EvalBPDirectEEUpdateSet(self, mol_set, Rr_cut, Ra_cut, Ree_cut, HasVdw=False):
        """Ragged batch in one fused evaluation; per-atom outputs are returned
        zero-padded to [nmol, MaxNAtoms] like TFMolManage.py:1260-1288."""
        self._check_cuts(Rr_cut, Ra_cut, Ree_cut)
        mols = mol_set.mols
        nmol, maxn = _padded(mols)
        Z = np.concatenate([np.asarray(m.atoms, dtype=np.int32) for m in mols])
        x = np.concatenate([np.asarray(m.coords, dtype=_F64) for m in mols])
        off = np.zeros(nmol + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(m.atoms) for m in mols])
        s = self._system(Z, off)
        o = s.energy_force(x, True, charges=True)
        pad = lambda a, w: np.stack([np.pad(a[off[m]:off[m + 1]], ((0, maxn - (off[m + 1] - off[m])),) + ((0, 0),) * (a.ndim - 1)) for m in range(nmol)])
        force = pad(o["force"], 3)
        if HasVdw:
            return (o["Etotal"], o["Ebp"], pad(o["Ebp_atom"], 1), o["Ecc"], o["Evdw"], o["dipole"],
                    pad(o["charge"], 1), force)
        return o["Etotal"], o["Ebp"], o["Ecc"], o["dipole"], pad(o["charge"], 1), force

    def EvalBPDirectEEUpdateSinglePeriodic(self, mol, Rr_cut, Ra_cut, Ree_cut, nreal, HasVdw=True,
                                           DoForce=True, DoCharge=False, lattice=None,
                                           reference_force=False):
        """Periodic cell (TFMolManage.py:1323-1358). Takes the real atoms and the
        lattice (mol.properties["Lattice"] if not given) instead of a tessellated
        molecule: images are generated on the device by minimum image. Returns
        (Etotal, force[1, nreal, 3]) or Etotal with DoForce=False."""
        self._check_cuts(Rr_cut, Ra_cut, Ree_cut)
        lat = lattice
        if lat is None:
            lat = np.asarray(mol.properties["Lattice"], dtype=_F64).reshape(3, 3)
        Z = np.ascontiguousarray(np.asarray(mol.atoms)[:nreal], dtype=np.int32)
        x = np.ascontiguousarray(np.asarray(mol.coords)[:nreal], dtype=_F64)
        s = self._system(Z, np.array([0, nreal], dtype=np.int64), np.asarray(lat, dtype=_F64))
        o = s.energy_force(x, DoForce, charges=DoCharge, reference_periodic_force=reference_force)
        if not DoForce:
            return o["Etotal"]
        if DoCharge:
            return o["Etotal"], o["force"].reshape(1, nreal, 3), o["charge"].reshape(1, nreal)
        return o["Etotal"], o["force"].reshape(1, nreal, 3)


def EnergyAndForce(manager, atoms, Rr_cut=None, Ra_cut=None, Ree_cut=None):
    """The closure the reference's samples hand to GeomOptimizer, VelocityVerlet
    and NudgedElasticBand (samples/test_tensormol01.py:61-69):
    f(x_, DoForce=True) -> (Etotal Hartree, F[N,3] J/mol/A), or Etotal only."""
    p = manager.Instances.p
    Rr = p["AN1_r_Rc"] if Rr_cut is None else Rr_cut
    Ra = p["AN1_a_Rc"] if Ra_cut is None else Ra_cut
    Re = p["EECutoffOff"] if Ree_cut is None else Ree_cut
    Z = np.ascontiguousarray(atoms, dtype=np.int32)
    manager._check_cuts(Rr, Ra, Re)
    sysm = manager._system(Z, np.array([0, len(Z)], dtype=np.int64))

    def EnAndForce(x_, DoForce=True):
        o = sysm.energy_force(np.asarray(x_, dtype=_F64), DoForce)
        if DoForce:
            return o["Etotal"][0], o["force"]
        return o["Etotal"][0]

    def system_for(x_):
        """The device system behind the closure, holding positions x_ (the
        device integrators in ``tensormol_gb300.md`` drive it directly)."""
        sysm.set_positions(np.asarray(x_, dtype=_F64))
        return sysm

    EnAndForce.system_for = system_for
    EnAndForce.model = manager.Instances   # lets drivers batch structures (tensormol_gb300.opt)
    return EnAndForce


class Mol:
    """Minimal molecule container with the reference's fields
    (Containers/Mol.py:7-23: atoms, coords, properties)."""

    def __init__(self, atoms=None, coords=None):
        self.atoms = np.asarray([] if atoms is None else atoms, dtype=np.int64)
        self.coords = np.asarray(np.zeros((0, 3)) if coords is None else coords, dtype=_F64)
        self.properties = {}

    def NAtoms(self):
        return int(self.atoms.shape[0])

    # -- XYZ text, the reference's format (Containers/Mol.py:268-360) -------
    def PropertyString(self):
        out = ""
        for prop, val in self.properties.items():
            out += ";;;" + prop + " " + str(val)
        return out

    def __str__(self, wprop=False):
        n = self.NAtoms()
        lines = str(n) + "\nComment: " + (self.PropertyString() if wprop else "") + "\n"
        rows = [_SYMBOLS[int(z)] + "   " + str(c[0]) + "  " + str(c[1]) + "  " + str(c[2])
                for z, c in zip(self.atoms, self.coords)]
        return lines + "\n".join(rows)

    def WriteXYZfile(self, fpath=".", fname="mol", mode="a", wprop=False):
        import os
        path = os.path.join(fpath, fname + ".xyz")
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        with open(path, mode) as f:
            for line in self.__str__(wprop).split("\n"):
                f.write(line + "\n")

    def FromXYZString(self, string):
        lines = string.split("\n")
        n = int(lines[0])
        if "Comment:" in lines[1]:
            for prop in lines[1].split("Comment:")[1].split(";;;"):
                s = prop.split()
                if len(s) >= 2:
                    try:
                        self.properties[s[0]] = float(s[1])
                    except ValueError:
                        self.properties[s[0]] = " ".join(s[1:])
        atoms, coords = [], []
        for i in range(n):
            t = lines[i + 2].split()
            atoms.append(_SYMBOLS.index(t[0]))
            coords.append([float(t[1]), float(t[2]), float(t[3])])
        self.atoms = np.array(atoms, dtype=np.int64)
        self.coords = np.array(coords, dtype=_F64)

    def ReadAtomsFromXYZFile(self, path):
        with open(path) as f:
            self.FromXYZString(f.read())


class MSet:
    """Minimal molecule set (Containers/Sets.py:17): a list of Mol."""

    def __init__(self, mols=None):
        self.mols = list(mols or [])

    def MaxNAtoms(self):
        return max(m.NAtoms() for m in self.mols)
