"""A minimal loopback i-PI server (for tests, benchmarks and checking a driver set-up without
i-PI): the server side of the exchange that the reference's client answers
(SOURCE/ipi.f90:33-198): STATUS, INIT, POSDATA, GETFORCE, EXIT.

`FakeIpiServer(frames)` listens on 127.0.0.1 (an ephemeral port) and, in a thread, sends
each frame (replica, h[9], hinv[9], positions[n, 3] in bohr) and collects the client's
FORCEREADY reply (energy, forces[n, 3], virial[9], extra text), then sends EXIT.
"""
import socket
import struct
import threading

import numpy as np


def _hdr(text):
    return text.encode().ljust(12)


class FakeIpiServer:
    """unix_dir/unix_name: listen on the unix socket <unix_dir>/ipi_<unix_name> (the client
    finds it through MBX_IPI_UNIX_DIR) instead of TCP."""

    def __init__(self, frames, init_text="params", unix_dir=None, unix_name=None):
        self.frames = frames
        self.init_text = init_text.encode()
        self.replies = []
        self.statuses = []
        self.error = None
        self.unix = unix_dir is not None
        if self.unix:
            import os
            self.path = os.path.join(unix_dir, "ipi_" + unix_name)
            self.sock = socket.socket(socket.AF_UNIX, socket.SOCK_STREAM)
            self.sock.bind(self.path)
            self.address = "unix:%s:0" % unix_name
        else:
            self.sock = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
            self.sock.bind(("127.0.0.1", 0))
        self.sock.listen(1)
        self.sock.settimeout(300)
        if not self.unix:
            self.port = self.sock.getsockname()[1]
            self.address = "inet:127.0.0.1:%d" % self.port
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _recv(self, conn, n):
        buf = b""
        while len(buf) < n:
            chunk = conn.recv(n - len(buf))
            if not chunk:
                raise ConnectionError("client closed the connection")
            buf += chunk
        return buf

    def _status(self, conn):
        conn.sendall(_hdr("STATUS"))
        s = self._recv(conn, 12).decode().strip()
        self.statuses.append(s)
        return s

    def _run(self):
        try:
            conn, _ = self.sock.accept()
            conn.settimeout(300)
            if not self.unix:
                conn.setsockopt(socket.IPPROTO_TCP, socket.TCP_NODELAY, 1)
            with conn:
                for replica, h, hinv, pos in self.frames:
                    if self._status(conn) == "NEEDINIT":
                        conn.sendall(_hdr("INIT") + struct.pack("<ii", replica, len(self.init_text)) + self.init_text)
                    assert self._status(conn) == "READY"
                    pos = np.ascontiguousarray(pos, np.float64)
                    conn.sendall(_hdr("POSDATA") + np.asarray(h, np.float64).tobytes() +
                                 np.asarray(hinv, np.float64).tobytes() + struct.pack("<i", pos.shape[0]) +
                                 pos.tobytes())
                    assert self._status(conn) == "HAVEDATA"
                    conn.sendall(_hdr("GETFORCE"))
                    assert self._recv(conn, 12).decode().strip() == "FORCEREADY"
                    pot = struct.unpack("<d", self._recv(conn, 8))[0]
                    nat = struct.unpack("<i", self._recv(conn, 4))[0]
                    f = np.frombuffer(self._recv(conn, 24 * nat), np.float64).reshape(nat, 3).copy()
                    vir = np.frombuffer(self._recv(conn, 72), np.float64).copy()
                    ln = struct.unpack("<i", self._recv(conn, 4))[0]
                    text = self._recv(conn, ln).decode()
                    self.replies.append(dict(energy=pot, natoms=nat, forces=f, virial=vir, text=text))
                conn.sendall(_hdr("EXIT"))
        except Exception as e:   # reported by the test
            self.error = e
        finally:
            self.sock.close()

    def join(self):
        self.thread.join(timeout=300)
