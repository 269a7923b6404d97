"""DCD trajectories (pdynamo_mirror_gb300/trajectory.py) against the record layout of pBabel's DCDWrite.c
(pBabel-1.9.0/extensions/csource/DCDWrite.c:62-269): header words, title records, the atom count and free-atom
index records, float32 coordinate records (all atoms first, free atoms afterwards when atoms are fixed), the
NFILE / NSTEP words rewritten after every frame, and the round trip through the reader; and the directory
trajectories (SystemGeometryTrajectory, pBabel-1.9.0/pBabel/SystemGeometryTrajectory.py): modes, frame order,
interpolation, expansion and superposition.  No GPU."""
import struct

import numpy as np
import pytest

from pdynamo_mirror_gb300 import DCDTrajectoryFileReader, DCDTrajectoryFileWriter, System


def _system(n=7, fixed=None):
    s = System([8, 1, 1, 8, 1, 1, 6][:n], np.arange(3 * n, dtype=float).reshape(n, 3) * 0.37)
    if fixed is not None:
        s.DefineFixedAtoms(fixed)
    return s


def test_header_layout_matches_dcdwrite(tmp_path):
    s = _system()
    w = DCDTrajectoryFileWriter(tmp_path / "a.dcd", s, title="water box frames", timeStep=0.0005, saveFrequency=5)
    w.WriteHeader()
    for k in range(3):
        w.WriteFrame(s.coordinates3 + k)
    w.Close()
    b = (tmp_path / "a.dcd").read_bytes()
    assert struct.unpack_from("<i", b, 0)[0] == 84 and b[4:8] == b"CORD"
    flags = struct.unpack_from("<23i", b, 8)
    assert flags[0] == 3 and flags[1] == 0 and flags[2] == 5 and flags[3] == 15   # NFILE, ISTART, NSAVC, NSTEP
    assert flags[8] == 0 and flags[10] == 0 and flags[19] == 34
    assert abs(struct.unpack("<f", struct.pack("<i", flags[9]))[0] - 0.0005) < 1e-10
    assert flags[20:] == (84, 164, 2)
    assert b[100:180].rstrip(b"\0") == b"water box frames" and b[180:195] == b"REMARKS Created"
    assert struct.unpack_from("<4i", b, 260) == (164, 4, 7, 4)
    # first coordinate record: x of all atoms as float32
    assert struct.unpack_from("<i", b, 276)[0] == 28
    np.testing.assert_array_equal(np.frombuffer(b, "<f4", 7, 280), s.coordinates3[:, 0].astype(np.float32))
    assert len(b) == 276 + 3 * 3 * (28 + 8)


def test_fixed_atoms_are_written_once(tmp_path):
    s = _system(fixed=[0, 2, 3])
    w = DCDTrajectoryFileWriter(tmp_path / "f.dcd", s)
    w.WriteHeader()
    frames = [s.coordinates3 + 0.1 * k for k in range(4)]
    for X in frames:
        w.WriteFrame(X)
    w.Close()
    b = (tmp_path / "f.dcd").read_bytes()
    flags = struct.unpack_from("<23i", b, 8)
    assert flags[8] == 3
    nb = struct.unpack_from("<i", b, 276)[0]
    assert nb == 16 and list(np.frombuffer(b, "<i4", 4, 280)) == [2, 5, 6, 7]   # free atoms, 1-based
    first = 276 + 16 + 8
    assert len(b) == first + 3 * (28 + 8) + 3 * 3 * (16 + 8)
    r = DCDTrajectoryFileReader(tmp_path / "f.dcd")
    assert len(r) == 4 and r.numberOfAtoms == 7 and list(r.atomIndices) == [1, 4, 5, 6]
    for k in range(4):
        expect = frames[k].copy()
        expect[[0, 2, 3]] = frames[0][[0, 2, 3]]   # fixed atoms keep their first-frame positions
        np.testing.assert_allclose(r.ReadFrame(k), expect.astype(np.float32), rtol=0, atol=0)


def test_round_trip_and_errors(tmp_path):
    s = _system(5)
    w = DCDTrajectoryFileWriter(tmp_path / "r.dcd", s, startingFrame=10, saveFrequency=2)
    w.WriteHeader()
    rng = np.random.default_rng(1)
    frames = [rng.normal(size=(5, 3)) * 10 for _ in range(6)]
    for X in frames:
        w.WriteFrame(X)
    w.Close()
    r = DCDTrajectoryFileReader(tmp_path / "r.dcd")
    assert (r.numberOfFrames, r.startingFrame, r.saveFrequency, r.numberOfSteps) == (6, 10, 2, 22)
    for k, X in enumerate(frames):
        np.testing.assert_array_equal(r.ReadFrame(k), X.astype(np.float32))
    with pytest.raises(IndexError):
        r.ReadFrame(6)
    (tmp_path / "bad.dcd").write_bytes(b"\0" * 300)
    with pytest.raises(ValueError):
        DCDTrajectoryFileReader(tmp_path / "bad.dcd")


# ---- directory trajectories (SystemGeometryTrajectory) ----
class _Owner:
    def __init__(self, X, fixed=None):
        self.coordinates3 = np.array(X, dtype=np.float64)
        self.fixedAtoms = fixed


def _rotation(angle, axis):
    a = np.asarray(axis, float) / np.linalg.norm(axis)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + np.sin(angle) * K + (1 - np.cos(angle)) * K @ K


def test_directory_trajectory_modes_and_frames(tmp_path):
    from pdynamo_mirror_gb300 import SystemGeometryTrajectory
    rng = np.random.default_rng(1)
    X = rng.normal(size=(7, 3))
    owner = _Owner(X)
    path = tmp_path / "traj"
    with pytest.raises(IOError):
        SystemGeometryTrajectory(path, owner, mode="r")
    t = SystemGeometryTrajectory(path, owner)           # new: "w"
    assert t.mode == "w" and t.isWritable and t.isReadable
    for k in range(3):
        owner.coordinates3 = X + k
        t.WriteOwnerData()
    assert len(t) == 3
    r = SystemGeometryTrajectory(path, owner)           # existing: "r"
    assert r.mode == "r" and len(r) == 3 and not r.isWritable
    with pytest.raises(IOError):
        r.WriteFrame(X)
    np.testing.assert_array_equal(r[2], X + 2)
    with pytest.raises(IndexError):
        r[3]
    seen = []
    while r.RestoreOwnerData():
        seen.append(owner.coordinates3.copy())
    assert len(seen) == 3 and np.array_equal(seen[1], X + 1)
    assert r.RestoreOwnerData(index=0) and np.array_equal(owner.coordinates3, X)
    a = SystemGeometryTrajectory(path, owner, mode="a")
    assert len(a) == 3
    a.WriteFrame(X - 1)
    assert len(SystemGeometryTrajectory(path, owner, mode="r")) == 4
    w = SystemGeometryTrajectory(path, owner, mode="w")  # write modes clear the frames
    assert len(w) == 0 and len(SystemGeometryTrajectory(path, owner, mode="r")) == 0
    f = tmp_path / "file"
    f.write_text("x")
    with pytest.raises(IOError):
        SystemGeometryTrajectory(f, owner)
    with pytest.raises(IOError):
        SystemGeometryTrajectory(tmp_path / "other", owner, mode="q")


def test_superposition_recovers_a_rigid_motion():
    from pdynamo_mirror_gb300.trajectory import rms_deviation, superimpose
    rng = np.random.default_rng(2)
    X = rng.normal(size=(12, 3)) * 3.0
    Y = X @ _rotation(1.1, [1, 2, -0.5]).T + np.array([4.0, -2.0, 9.0])
    assert rms_deviation(Y, X) > 1.0
    np.testing.assert_allclose(superimpose(Y, X), X, atol=1e-12)
    w = rng.uniform(0.5, 2.0, size=12)
    np.testing.assert_allclose(superimpose(Y, X, w), X, atol=1e-12)
    assert rms_deviation(superimpose(Y + rng.normal(scale=0.1, size=Y.shape), X), X) < 0.2


def test_linear_interpolation_and_expansion(tmp_path):
    from pdynamo_mirror_gb300 import SystemGeometryTrajectory
    rng = np.random.default_rng(3)
    X0 = rng.normal(size=(6, 3)) * 2.0
    Xn = X0 + rng.normal(scale=0.3, size=X0.shape)
    # fixed atoms: plain linear interpolation, no superposition
    owner = _Owner(X0, fixed=[0])
    t = SystemGeometryTrajectory.LinearlyInterpolate(tmp_path / "i", owner, 5, X0, Xn)
    assert len(t) == 5
    for k in range(5):
        np.testing.assert_allclose(t[k], X0 + (Xn - X0) * k / 4.0, atol=1e-12)
    # expansion: ninsert frames between each pair, the old frames kept at their new places
    t.LinearlyExpand(2)
    assert len(t) == 13
    for k in range(13):
        np.testing.assert_allclose(t[k], X0 + (Xn - X0) * k / 12.0, atol=1e-12)
    # without fixed atoms the end point is superimposed on the start first: a rigidly moved copy interpolates
    # to the start structure everywhere
    owner = _Owner(X0)
    Y = X0 @ _rotation(0.7, [0, 1, 1]).T + 3.0
    t = SystemGeometryTrajectory.LinearlyInterpolate(tmp_path / "j", owner, 3, X0, Y)
    for k in range(3):
        np.testing.assert_allclose(t[k], X0, atol=1e-12)


def test_trajectory_superimpose(tmp_path):
    from pdynamo_mirror_gb300 import SystemGeometryTrajectory
    rng = np.random.default_rng(4)
    X = rng.normal(size=(9, 3)) * 2.0
    owner = _Owner(X)
    t = SystemGeometryTrajectory(tmp_path / "s", owner, mode="w")
    for k in range(4):
        t.WriteFrame(X @ _rotation(0.3 * k, [1, 0, 1]).T + k)
    res = t.Superimpose()
    assert len(res) == 4 and all(after <= before + 1e-12 for before, after in res) and res[3][0] > 1.0
    for k in range(4):
        np.testing.assert_allclose(t[k], X, atol=1e-12)
    np.testing.assert_array_equal(owner.coordinates3, X)
