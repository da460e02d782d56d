"""The i-PI client (tensormol_gb300.ipi, the reference's
Interfaces/TMIPIinterface.py:19-61) driving the device EnergyAndForce closure:
a scripted i-PI server on the other end of a socket pair moves a 60-atom water
cluster for three steps along the forces it receives (positions in bohr,
forces in Hartree/bohr on the wire) and each answer is checked against the
FP64 oracle at the positions sent (1e-5 eV/atom, 1e-4 eV/A)."""
import socket
import threading

import numpy as np
import pytest

from oracle import reference as orc
from tensormol_gb300 import systems
from tensormol_gb300.params import BOHRPERA, EV_PER_HARTREE, PARAMS, descriptor_width

pytestmark = pytest.mark.gpu


def _server(sock, x_bohr, nsteps, log):
    def hdr(t):
        sock.sendall(t.encode().ljust(12))

    def recv(n):
        b = b""
        while len(b) < n:
            b += sock.recv(n - len(b))
        return b
    x = x_bohr.copy()
    for _ in range(nsteps):
        hdr("STATUS")
        assert recv(12).decode().strip() == "READY"
        hdr("POSDATA")
        sock.sendall(np.eye(3).tobytes() + np.eye(3).tobytes() + np.int32(len(x)).tobytes()
                     + x.tobytes())
        hdr("STATUS")
        assert recv(12).decode().strip() == "HAVEDATA"
        hdr("GETFORCE")
        assert recv(12).decode().strip() == "FORCEREADY"
        E = np.frombuffer(recv(8), np.float64)[0]
        n = int(np.frombuffer(recv(4), np.int32)[0])
        F = np.frombuffer(recv(24 * n), np.float64).reshape(-1, 3).copy()
        recv(72 + 4)
        log.append((x.copy(), E, F))
        x = x + 2.0 * F            # a steepest-descent step, bohr per Hartree/bohr
    hdr("EXIT")


def test_ipi_drives_the_device_path():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tensormol_gb300 import ipi
    from tensormol_gb300.model import BPEEModel, EnergyAndForce, TFMolManage
    p = dict(PARAMS)
    p["NeuronType"] = "sigmoid_with_param"
    W = systems.random_weights([1, 8], descriptor_width(2), seed=7)
    w = systems.water_cluster_60(seed=0)
    manager = TFMolManage(BPEEModel([1, 8], W, params=p, precision="fp32"))
    ef = EnergyAndForce(manager, w.Z)
    a, b = socket.socketpair()
    log = []
    t = threading.Thread(target=_server, args=(b, w.x * BOHRPERA, 3, log))
    t.start()
    ipi.TMIPIManger(ef, sock=a).md_run()
    t.join(timeout=30)
    assert len(log) == 3
    om = orc.Model([1, 8], W, p)
    for x_bohr, E, F in log:
        x = x_bohr / BOHRPERA
        ref = orc.OpenSystemOracle(om, x, w.Z, w.offsets).terms(x)
        dE = abs(E - ref["Etotal"][0]) * EV_PER_HARTREE / w.natoms
        # wire forces are -dE/dx in Hartree/bohr; the oracle's gradient is per A
        dF = np.abs(F - (-ref["gradient"] / BOHRPERA)).max() * EV_PER_HARTREE * BOHRPERA
        assert dE < 1e-5 and dF < 1e-4, (dE, dF)
    assert np.abs(log[2][0] - log[0][0]).max() > 1e-4   # the server did move the atoms
