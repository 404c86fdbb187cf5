"""i-PI driver mode (mbx_ipi_run_callback) on the CPU: the protocol exchange of the
reference's client (SOURCE/ipi.f90:33-198) against a fake i-PI server, with a Python force
function.  Checked bit for bit: the unit factors (the reference's single-precision REAL
constants promoted to double), the cell transpose, the force and virial layouts, the
dipole text, and the STATUS answers through two replicas and three frames."""
import numpy as np
import pytest

from mbx import capi
from mbx.ipi_loopback import FakeIpiServer

BOHR = np.float64(np.float32(0.52917721067))
E_AU = np.float64(np.float32(3.8087989e-06))
RATIO = np.float64(np.float32(np.float64(np.float32(418.6799938)) / 418.4))


def _frames(rng, nat=6):
    out = []
    for k, replica in enumerate((0, 0, 1)):
        h = rng.normal(0.0, 0.3, 9) + np.array([30.0, 0, 0, 0, 31.0, 0, 0, 0, 32.0])
        hinv = np.linalg.inv(h.reshape(3, 3)).ravel()
        pos = rng.uniform(0.0, 25.0, (nat, 3))
        out.append((replica, h, hinv, pos))
    return out


@pytest.fixture(scope="module")
def lib():
    try:
        return capi.load()
    except capi.MbxError as e:
        pytest.skip(str(e))


def test_ipi_protocol_and_units(lib):
    rng = np.random.default_rng(11)
    frames = _frames(rng)
    seen = []

    def force(replica, cell, xyz):
        seen.append((replica, cell, xyz))
        k = 0.7
        e = 0.5 * k * float((xyz ** 2).sum())
        f = -k * xyz
        st = np.arange(1.0, 10.0) * (replica + 1)
        md = np.arange(xyz.shape[0] // 3 * 3, dtype=np.float64).reshape(-1, 3) * 0.25 + replica
        return e, f, st, md

    srv = FakeIpiServer(frames)
    rc, steps, err = capi.ipi_run_callback(srv.address, force)
    srv.join()
    assert srv.error is None, srv.error
    assert rc == 0 and steps == 3, (rc, steps, err)
    # NEEDINIT before each frame (GETFORCE clears the initialisation), READY, HAVEDATA
    assert srv.statuses == ["NEEDINIT", "READY", "HAVEDATA"] * 3
    for (replica, h, _, pos), (rep_seen, cell, xyz), reply in zip(frames, seen, srv.replies):
        assert rep_seen == replica
        # positions and cell to Angstrom with the single-precision factor; cell = transpose(h)
        np.testing.assert_array_equal(xyz, pos * BOHR)
        want_cell = np.array([h[b + 3 * a] for b in range(3) for a in range(3)]) * BOHR
        np.testing.assert_array_equal(cell, want_cell)
        e, f, st, md = 0.5 * 0.7 * float((xyz ** 2).sum()), -0.7 * xyz, np.arange(1.0, 10.0) * (replica + 1), None
        assert reply["energy"] == e * E_AU * RATIO
        np.testing.assert_array_equal(reply["forces"], f * E_AU * BOHR * RATIO)
        want_vir = np.array([st[b + 3 * a] for b in range(3) for a in range(3)]) * E_AU * RATIO
        np.testing.assert_array_equal(reply["virial"], want_vir)
        vals = np.array([float(t) for t in reply["text"].split()])
        np.testing.assert_array_equal(vals, np.arange(6, dtype=np.float64) * 0.25 + replica)
        assert reply["natoms"] == pos.shape[0]


def test_ipi_max_steps_and_errors(lib):
    rng = np.random.default_rng(12)
    srv = FakeIpiServer(_frames(rng))

    def force(replica, cell, xyz):
        return 0.0, np.zeros_like(xyz), np.zeros(9), np.zeros((xyz.shape[0] // 3, 3))

    rc, steps, err = capi.ipi_run_callback(srv.address, force, max_steps=1)
    assert rc == 0 and steps == 1
    srv.join()   # the server sees the connection close after the first reply
    # no server listening: a connection error, not a crash
    rc, steps, err = capi.ipi_run_callback("inet:127.0.0.1:1", force)
    assert rc == capi.ERR_ARG and steps == 0 and "connect" in err
    rc, _, err = capi.ipi_run_callback("nonsense", force)
    assert rc == capi.ERR_ARG and "address" in err


def test_polar_params_for_cell_matches_systems(lib):
    for cell in ([19.73, 0, 0, 0, 19.73, 0, 0, 0, 19.73], [49.7, 0, 0, 0, 49.7, 0, 0, 0, 49.7],
                 [12.4, 0, 0, 2.0, 12.0, 0, 1.0, -1.5, 13.0]):
        got = capi.polar_params_for_cell(cell)
        from mbx import systems
        want = systems.polar_params_for(np.array(cell, np.float64))
        np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)


def test_ipi_unix_socket(lib, tmp_path, monkeypatch):
    """The unix-socket form of the address (the reference's /tmp/ipi_<name>; the directory
    from MBX_IPI_UNIX_DIR here): the same exchange as over TCP."""
    import os
    monkeypatch.setenv("MBX_IPI_UNIX_DIR", str(tmp_path))
    rng = np.random.default_rng(13)
    frames = _frames(rng)
    srv = FakeIpiServer(frames, unix_dir=str(tmp_path), unix_name="t%d" % os.getpid())

    def force(replica, cell, xyz):
        return 0.5 * float((xyz ** 2).sum()), -xyz, np.zeros(9), np.zeros((xyz.shape[0] // 3, 3))

    rc, steps, err = capi.ipi_run_callback(srv.address, force)
    srv.join()
    assert srv.error is None, srv.error
    assert rc == 0 and steps == 3, (rc, steps, err)
    assert srv.statuses == ["NEEDINIT", "READY", "HAVEDATA"] * 3
    for (_, _, _, pos), reply in zip(frames, srv.replies):
        np.testing.assert_array_equal(reply["forces"], -(pos * BOHR) * E_AU * BOHR * RATIO)
    # no socket there: a connection error naming the path
    rc, _, err = capi.ipi_run_callback("unix:absent%d:0" % os.getpid(), force)
    assert rc == capi.ERR_ARG and str(tmp_path) in err
