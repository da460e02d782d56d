"""Host-side formats next to the path: the i-PI socket client, XYZ text and
trajectory files, and trained-weight loading by the reference's variable
names. CPU only (stand-in energy functions where a GPU would be needed)."""
import socket
import threading

import numpy as np

from tensormol_gb300 import ipi, systems
from tensormol_gb300.model import Mol
from tensormol_gb300.params import BOHRPERA, JOULEPERHARTREE, descriptor_width
from tensormol_gb300.weights import load_tensormol_weights, tensormol_names


def _fake_server(sock, x_bohr, out):
    def hdr(t):
        sock.sendall(t.encode().ljust(12))

    def recv(n):
        b = b""
        while len(b) < n:
            b += sock.recv(n - len(b))
        return b
    hdr("STATUS")
    out["status1"] = recv(12).decode().strip()
    hdr("INIT")
    sock.sendall(np.int32(0).tobytes() + np.int32(3).tobytes() + b"abc")
    hdr("POSDATA")
    sock.sendall(np.eye(3).tobytes() + np.eye(3).tobytes() + np.int32(len(x_bohr)).tobytes()
                 + x_bohr.tobytes())
    hdr("STATUS")
    out["status2"] = recv(12).decode().strip()
    hdr("GETFORCE")
    out["ready"] = recv(12).decode().strip()
    out["E"] = np.frombuffer(recv(8), np.float64)[0]
    n = np.frombuffer(recv(4), np.int32)[0]
    out["F"] = np.frombuffer(recv(24 * n), np.float64).reshape(-1, 3)
    out["vir"] = np.frombuffer(recv(72), np.float64)
    out["extra"] = np.frombuffer(recv(4), np.int32)[0]
    hdr("EXIT")


def test_ipi_client_units_and_messages():
    x = np.array([[0.0, 0.0, 0.0], [0.0, 0.0, 0.96], [0.9, 0.0, -0.3]])
    seen = {}

    def eff(pos):                       # E in Hartree, F in J/mol/A
        seen["x"] = pos.copy()
        return 0.25, -JOULEPERHARTREE * 0.1 * pos
    a, b = socket.socketpair()
    out = {}
    t = threading.Thread(target=_fake_server, args=(b, x * BOHRPERA, out))
    t.start()
    ipi.TMIPIManger(eff, sock=a).md_run()
    t.join(timeout=10)
    np.testing.assert_allclose(seen["x"], x, rtol=1e-14)
    assert out["status1"] == "READY" and out["status2"] == "HAVEDATA" and out["ready"] == "FORCEREADY"
    assert out["E"] == 0.25 and out["extra"] == 0 and not out["vir"].any()
    np.testing.assert_allclose(out["F"], -0.1 * x / BOHRPERA, rtol=1e-14)   # Hartree / bohr


def test_xyz_round_trip_and_file(tmp_path):
    w = systems.water(3, seed=1)
    m = Mol(w.Z, w.x)
    m.properties["energy"] = -76.4
    m.WriteXYZfile(str(tmp_path), "traj", "a", True)
    m.WriteXYZfile(str(tmp_path), "traj", "a", True)
    text = (tmp_path / "traj.xyz").read_text()
    frames = text.strip().split("\n" + str(len(w.Z)) + "\n")
    assert len(frames) == 2 and text.startswith("9\nComment: ;;;energy -76.4\nO   ")
    m2 = Mol()
    m2.FromXYZString(text)
    assert np.array_equal(m2.atoms, w.Z) and np.allclose(m2.coords, w.x, rtol=0, atol=1e-12)
    assert m2.properties["energy"] == -76.4


def test_weights_by_reference_names():
    W = systems.random_weights([1, 8], descriptor_width(2), hidden=(64, 32), seed=3)
    names = tensormol_names(W)
    assert "EnergyNet/8_hidden2/biaseslayer1" in names
    assert "DipoleNet/1_regression_linear_charge/weights" in names
    names = {k + ":0": v for k, v in names.items()}       # TensorFlow tensor-name form
    back = load_tensormol_weights(names, [1, 8], 2)
    for net in ("E", "Q"):
        for e in (1, 8):
            for (W0, b0), (W1, b1) in zip(W[net][e], back[net][e]):
                assert np.array_equal(W0, W1) and np.array_equal(b0, b1)


def test_xyz_text_matches_the_reference(tmp_path):
    """The XYZ text of Mol.__str__ / WriteXYZfile equals what the reference's
    own Mol.__str__ and PropertyString produce for the same molecule
    (tests/golden/make_golden_xyz.py), with and without the property line."""
    import ast
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "xyz.npz"))
    for name in ("water60", "water60_props", "chno0"):
        m = Mol(g[name + "_Z"], g[name + "_x"])
        m.properties.update(ast.literal_eval(str(g[name + "_props"])))
        wprop = bool(g[name + "_wprop"])
        assert m.__str__(wprop) == str(g[name + "_text"]), name
        m.WriteXYZfile(str(tmp_path), name, mode="w", wprop=wprop)
        assert (tmp_path / (name + ".xyz")).read_text() == str(g[name + "_text"]) + "\n", name
