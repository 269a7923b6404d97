"""DCD trajectories (pdynamo_mirror_gb300/trajectory.py) against the record layout of pBabel's DCDWrite.c
(pBabel-1.9.0/extensions/csource/DCDWrite.c:62-269): header words, title records, the atom count and free-atom
index records, float32 coordinate records (all atoms first, free atoms afterwards when atoms are fixed), the
NFILE / NSTEP words rewritten after every frame, and the round trip through the reader.  No GPU."""
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
