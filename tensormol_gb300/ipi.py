"""i-PI socket client for the energy/force path.

Follows the reference's client (Interfaces/TMIPIinterface.py:8-61): 12-byte
message headers; on POSDATA it reads the cell (h and its inverse, 9 float64
each, bohr), the atom count (int32) and the positions (float64, bohr),
converts them to Angstrom, calls ``EnergyForceField(x) -> (E Hartree,
F J/mol/A)``, and on GETFORCE answers FORCEREADY, the energy (Hartree), the
atom count, the forces in Hartree/bohr, a zero virial and an empty extra
string. Differences from the reference's code, which targets Python 2: bytes
on the wire, every read completes its full length, and the INIT and EXIT
messages of the i-PI protocol are handled rather than raising.
"""
from __future__ import annotations

import socket

import numpy as np

from .params import BOHRPERA, JOULEPERHARTREE

HDRLEN = 12


def _recvall(sock, n):
    buf = bytearray()
    while len(buf) < n:
        chunk = sock.recv(n - len(buf))
        if not chunk:
            raise ConnectionError("i-PI server closed the connection")
        buf += chunk
    return bytes(buf)


def _header(text):
    return text.encode("ascii").ljust(HDRLEN)


class TMIPIManger:
    def __init__(self, EnergyForceField=None, TCP_IP="localhost", TCP_PORT=31415, sock=None):
        self.EnergyForceField = EnergyForceField
        self.hasdata = False
        self.s = sock
        if self.s is None:
            self.s = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
            self.s.connect((TCP_IP, TCP_PORT))
        self.energy = 0.0
        self.force = None
        self.natom = 0

    def md_run(self):
        """Serve the server's requests until it sends EXIT or disconnects."""
        while True:
            try:
                msg = _recvall(self.s, HDRLEN).decode("ascii").strip()
            except ConnectionError:
                return
            if msg == "STATUS":
                self.s.sendall(_header("HAVEDATA" if self.hasdata else "READY"))
            elif msg == "INIT":
                _recvall(self.s, 4)                                    # bead index
                n = int(np.frombuffer(_recvall(self.s, 4), np.int32)[0])
                _recvall(self.s, n)                                    # init string
            elif msg == "POSDATA":
                _recvall(self.s, 9 * 8)                                # cell h (bohr)
                _recvall(self.s, 9 * 8)                                # cell h^-1
                natom = int(np.frombuffer(_recvall(self.s, 4), np.int32)[0])
                pos = np.frombuffer(_recvall(self.s, 3 * natom * 8), np.float64)
                position = (pos / BOHRPERA).reshape((-1, 3))
                energy, force = self.EnergyForceField(position)
                self.energy = float(energy)
                self.force = np.ascontiguousarray(np.asarray(force, dtype=np.float64)
                                                  / JOULEPERHARTREE / BOHRPERA)
                self.natom = natom
                self.hasdata = True
            elif msg == "GETFORCE":
                self.s.sendall(_header("FORCEREADY"))
                self.s.sendall(np.float64(self.energy).tobytes())
                self.s.sendall(np.int32(self.natom).tobytes())
                self.s.sendall(self.force.tobytes())
                self.s.sendall(np.zeros((3, 3)).tobytes())
                self.s.sendall(np.int32(0).tobytes())
                self.hasdata = False
            elif msg == "EXIT":
                return
            else:
                raise Exception("wrong message from server")
