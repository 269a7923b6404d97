"""DCD trajectories of a System's coordinates (CHARMM format, as pDynamo's pBabel writes and reads them).

DCDTrajectoryFileWriter restates pBabel.DCDTrajectoryFileWriter (pBabel-1.9.0/extensions/pyrex/
pBabel.DCDTrajectoryFileWriter.pyx) over the record layout of DCDWrite_Header and DCDWrite_Frame
(pBabel-1.9.0/extensions/csource/DCDWrite.c:62-269):
  header   int32 84 | "CORD" | 20 control words (NFILE, ISTART, NSAVC, NSTEP, ..., the fixed-atom count, the time step
           as float32, the unit-cell flag, CHARMM version 34) and the next record's markers 84, 164, 2 (title lines) |
           80-byte title | 80-byte "REMARKS Created ..." line | int32 164; then the atom count record and, with fixed
           atoms, the 1-based indices of the free atoms;
  frame    x, y, z as float32 records of all atoms for the first frame and of the free atoms only afterwards;
           after every frame NFILE (byte 8) and NSTEP (byte 20) are rewritten.
DCDTrajectoryFileReader reads such files back (fixed atoms take their first-frame positions).
SystemGeometryTrajectory restates pBabel's directory trajectories (pBabel-1.9.0/pBabel/SystemGeometryTrajectory.py):
one file per frame, fopen-style modes, linear interpolation and expansion, superposition.  Host-side I/O: the
dynamics driver copies the replica it saves from the device.
"""

import os, struct, time

import numpy as np

CHARMM_VERSION = 34      # DCDWrite.c:23
NFILE_POS, NSTEP_POS = 8, 20   # DCDWrite.c:26-27


def _record(f, payload):
    f.write(struct.pack("<i", len(payload)))
    f.write(payload)
    f.write(struct.pack("<i", len(payload)))


class DCDTrajectoryFileWriter:
    """Writes frames of `owner` (a System) to `path`.  Fixed atoms (System.DefineFixedAtoms) are written once."""

    def __init__(self, path, owner, title="", timeStep=0.001, saveFrequency=1, startingFrame=0):
        self.path, self.owner, self.title = str(path), owner, title or ""
        self.timeStep, self.saveFrequency, self.startingFrame = float(timeStep), int(saveFrequency), int(startingFrame)
        self.numberOfAtoms = len(owner.atomicNumbers)
        fixed = set(getattr(owner, "fixedAtoms", None) or [])
        self.atomIndices = [i for i in range(self.numberOfAtoms) if i not in fixed] if fixed else None
        self.numberOfFrames = 0
        self.isOpen = False
        self.Open()

    def __len__(self):
        return self.numberOfFrames

    def Open(self):
        if not self.isOpen:
            self._f = open(self.path, "wb")
            self.isOpen = True

    def Close(self):
        if self.isOpen:
            self._f.close()
            self.isOpen = False

    def WriteHeader(self):
        """DCDWrite_Header (DCDWrite.c:147-200)."""
        f = self._f
        f.write(struct.pack("<i", 84))
        f.write(b"CORD")
        flags = [0] * 23
        flags[1], flags[2] = self.startingFrame, self.saveFrequency
        flags[8] = (self.numberOfAtoms - len(self.atomIndices)) if self.atomIndices is not None else 0
        flags[9] = struct.unpack("<i", struct.pack("<f", self.timeStep))[0]
        flags[10] = 0                      # no unit cell: the systems here are not periodic
        flags[19] = CHARMM_VERSION
        flags[20], flags[21], flags[22] = 84, 164, 2
        f.write(struct.pack("<23i", *flags))
        f.write(self.title.encode("ascii", "replace")[:79].ljust(80, b"\0"))
        f.write(time.strftime("REMARKS Created %d %B, %Y at %H:%M").encode("ascii")[:79].ljust(80, b"\0"))
        f.write(struct.pack("<i", 164))
        _record(f, struct.pack("<i", self.numberOfAtoms))
        if self.atomIndices is not None and len(self.atomIndices) > 0:
            _record(f, (np.asarray(self.atomIndices, dtype="<i4") + 1).tobytes())   # 1-based (DCDHandle.c:151)

    def WriteFrame(self, coordinates3):
        """DCDWrite_Frame / DCDWrite_Step (DCDWrite.c:62-118, 236-269) for coordinates [n_atoms, 3] in Angstrom."""
        X = np.asarray(coordinates3, dtype=np.float64).reshape(self.numberOfAtoms, 3)
        self.numberOfFrames += 1
        step = self.startingFrame + self.numberOfFrames * self.saveFrequency
        if self.numberOfFrames > 1 and self.atomIndices is not None and len(self.atomIndices) > 0:
            X = X[self.atomIndices]
        f = self._f
        for k in range(3):
            _record(f, np.ascontiguousarray(X[:, k], dtype="<f4").tobytes())
        f.seek(NFILE_POS)
        f.write(struct.pack("<i", self.numberOfFrames))
        f.seek(NSTEP_POS)
        f.write(struct.pack("<i", step))
        f.seek(0, os.SEEK_END)
        f.flush()

    def WriteOwnerData(self):
        """A frame of the owner's current coordinates (pBabel.DCDTrajectoryFileWriter.WriteOwnerData)."""
        self.WriteFrame(self.owner.coordinates3)

    def WriteFooter(self):
        pass


class DCDTrajectoryFileReader:
    """Reads a DCD file written as above (little-endian, no unit cell): header fields, then frames [n_atoms, 3]
    (float64, Angstrom); with fixed atoms the later frames hold only the free atoms and the fixed ones keep their
    first-frame positions (pBabel's DCDRead restores them the same way)."""

    def __init__(self, path):
        self.path = str(path)
        with open(self.path, "rb") as f:
            data = f.read()
        self._data = data
        n0, = struct.unpack_from("<i", data, 0)
        if n0 != 84 or data[4:8] not in (b"CORD", b"VELD"):
            raise ValueError("Not a DCD file written in this layout: %s" % self.path)
        flags = struct.unpack_from("<23i", data, 8)
        self.numberOfFrames, self.startingFrame, self.saveFrequency, self.numberOfSteps = flags[0], flags[1], flags[2], flags[3]
        self.numberOfFixedAtoms = flags[8]
        self.timeStep = struct.unpack("<f", struct.pack("<i", flags[9]))[0]
        self.hasUnitCell, self.charmmVersion = flags[10] != 0, flags[19]
        if self.hasUnitCell:
            raise ValueError("DCD files with a unit cell are not read here")
        pos = 8 + 92
        self.title = data[pos:pos + 80].split(b"\0")[0].decode("ascii", "replace")
        self.remarks = data[pos + 80:pos + 160].split(b"\0")[0].decode("ascii", "replace")
        pos += 160 + 4
        self.numberOfAtoms, = struct.unpack_from("<i", data, pos + 4)
        pos += 12
        self.atomIndices = None
        if self.numberOfFixedAtoms > 0:
            nb, = struct.unpack_from("<i", data, pos)
            self.atomIndices = np.frombuffer(data, dtype="<i4", count=nb // 4, offset=pos + 4) - 1
            pos += nb + 8
        self._first = pos
        self._first_size = 3 * (4 * self.numberOfAtoms + 8)
        nfree = self.numberOfAtoms if self.atomIndices is None else len(self.atomIndices)
        self._size = 3 * (4 * nfree + 8)
        self._frame0 = None

    def __len__(self):
        return self.numberOfFrames

    def _read_xyz(self, pos, n):
        out = np.empty((n, 3))
        for k in range(3):
            nb, = struct.unpack_from("<i", self._data, pos)
            if nb != 4 * n:
                raise ValueError("Bad record in %s" % self.path)
            out[:, k] = np.frombuffer(self._data, dtype="<f4", count=n, offset=pos + 4)
            pos += nb + 8
        return out

    def ReadFrame(self, frame):
        """Coordinates of frame `frame` (0-based) as [n_atoms, 3] float64."""
        if not 0 <= frame < self.numberOfFrames:
            raise IndexError("frame %d of %d" % (frame, self.numberOfFrames))
        if self._frame0 is None:
            self._frame0 = self._read_xyz(self._first, self.numberOfAtoms)
        if frame == 0 or self.atomIndices is None:
            if frame == 0:
                return self._frame0.copy()
            return self._read_xyz(self._first + self._first_size + (frame - 1) * self._size, self.numberOfAtoms)
        X = self._frame0.copy()
        X[self.atomIndices] = self._read_xyz(self._first + self._first_size + (frame - 1) * self._size, len(self.atomIndices))
        return X


# ---------------------------------------------------------------------------------------------------------------------
# Directory trajectories (pBabel-1.9.0/pBabel/SystemGeometryTrajectory.py): one file per frame in a directory, opening
# modes as C's fopen.  The reference pickles pCore Coordinates3 objects ("frame<n>.pkl"); here each frame is an
# [n_atoms, 3] float64 array in NumPy's .npy format ("frame<n>.npy", read without unpickling).

_FRAME_PREFIX, _FRAME_POSTFIX = "frame", ".npy"
_READABLE_MODES = ("a+", "r", "r+", "w", "w+")   # SystemGeometryTrajectory.py:36-38
_TRAJECTORY_MODES = ("a", "a+", "r", "r+", "w", "w+")
_WRITABLE_MODES = ("a", "a+", "r+", "w", "w+")


def rms_deviation(x, reference, weights=None):
    """Weighted RMS deviation between two [n, 3] coordinate sets (Coordinates3.RMSDeviation)."""
    w = np.ones(len(x)) if weights is None else np.asarray(weights, dtype=np.float64)
    d = ((np.asarray(x) - np.asarray(reference)) ** 2).sum(1)
    return float(np.sqrt((w * d).sum() / w.sum()))


def superimpose(x, reference, weights=None):
    """x rotated and translated onto reference by the weighted least-squares fit (Coordinates3.Superimpose), from
    the singular value decomposition of the weighted covariance (Kabsch, Acta Cryst. A32, 922 (1976))."""
    x, r = np.asarray(x, dtype=np.float64), np.asarray(reference, dtype=np.float64)
    w = np.ones(len(x)) if weights is None else np.asarray(weights, dtype=np.float64)
    cx, cr = (w[:, None] * x).sum(0) / w.sum(), (w[:, None] * r).sum(0) / w.sum()
    H = ((x - cx) * w[:, None]).T @ (r - cr)
    U, _, Vt = np.linalg.svd(H)
    D = np.diag([1.0, 1.0, np.sign(np.linalg.det(Vt.T @ U.T)) or 1.0])
    R = Vt.T @ D @ U.T
    return (x - cx) @ R.T + cr


class SystemGeometryTrajectory:
    """A trajectory of system geometries stored as a directory of frames (SystemGeometryTrajectory.py:43)."""

    def __init__(self, path, owner, mode=None):
        self.path, self.owner, self.mode = str(path), owner, mode
        self.frames, self.position = 0, -1
        self.isReadable = self.isWritable = False
        self.Open()

    def __len__(self):
        return self.frames

    def __getitem__(self, index):
        if index < 0 or index >= len(self):
            raise IndexError(index)
        return self.ReadFrame(frame=index)

    def _frame_path(self, f):
        return os.path.join(self.path, _FRAME_PREFIX + "{:d}".format(f) + _FRAME_POSTFIX)

    def _existing(self):
        n = []
        for name in os.listdir(self.path):
            if name.startswith(_FRAME_PREFIX) and name.endswith(_FRAME_POSTFIX):
                n.append(name)
        return n

    def Open(self):
        """Open (SystemGeometryTrajectory.py:161-192): "r" by default for an existing trajectory, "w" otherwise;
        write modes clear the frames of an existing trajectory."""
        if self.mode not in (None,) + _TRAJECTORY_MODES:
            raise IOError("Unrecognized mode: " + str(self.mode) + ".")
        exists = os.access(self.path, os.F_OK)
        if exists:
            if not os.path.isdir(self.path):
                raise IOError("Trajectory exists that is not a directory.")
            if self.mode is None:
                self.mode = "r"
        else:
            if self.mode is None:
                self.mode = "w"
            elif self.mode in ("r", "r+"):
                raise IOError("Read mode specified for a trajectory that does not exist.")
            os.mkdir(self.path)
        self.isReadable, self.isWritable = self.mode in _READABLE_MODES, self.mode in _WRITABLE_MODES
        if self.isReadable and not os.access(self.path, os.R_OK):
            raise IOError("Read mode specified for a trajectory that is unreadable.")
        if self.isWritable and not os.access(self.path, os.W_OK):
            raise IOError("Write mode specified for a trajectory that is unwriteable.")
        if exists:
            names = self._existing()
            if self.mode in ("w", "w+"):
                for name in names:
                    os.remove(os.path.join(self.path, name))
            else:
                self.frames = len(names)

    def Close(self):
        pass

    def ReadHeader(self):
        return {}

    def ReadFooter(self):
        return {}

    def WriteHeader(self, **keywordArguments):
        pass

    def WriteFooter(self):
        pass

    def ReadFrame(self, frame=None, identifier=None, instance=None):
        """Coordinates [n_atoms, 3] of a frame."""
        if not self.isReadable:
            raise IOError("Reading from trajectory that is not readable.")
        return np.load(self._frame_path(frame), allow_pickle=False)

    def WriteFrame(self, data, frame=None, identifier=None):
        """Write coordinates as frame `frame` (the next one when None)."""
        if not self.isWritable:
            raise IOError("Writing to trajectory that is not writeable.")
        f = self.frames if frame is None else int(frame)
        np.save(self._frame_path(f), np.ascontiguousarray(data, dtype=np.float64).reshape(-1, 3), allow_pickle=False)
        if frame is None:
            self.frames += 1

    def WriteOwnerData(self, index=-1):
        self.WriteFrame(self.owner.coordinates3, frame=index if index >= 0 else None)

    def RestoreOwnerData(self, index=-1):
        """Copy a frame (index >= 0) or the next frame into the owner's coordinates; False past the last frame."""
        data = None
        if index >= 0:
            data = self.ReadFrame(frame=index)
            self.position = index + 1
        else:
            self.position += 1
            if self.position >= self.frames:
                self.position = -1
            else:
                data = self.ReadFrame(frame=self.position)
        if data is None:
            return False
        self.owner.coordinates3 = np.array(data, dtype=np.float64)
        return True

    def _has_fixed_atoms(self):
        return bool(getattr(self.owner, "fixedAtoms", None))

    def LinearlyExpand(self, ninsert):
        """Insert ninsert linearly interpolated frames between each pair of frames (SystemGeometryTrajectory.py:70-118);
        without fixed atoms every frame is first superimposed on frame 0."""
        if not self.isWritable:
            raise IOError("Writing to trajectory that is not writeable.")
        if ninsert <= 0 or self.frames <= 1:
            return
        fixed = self._has_fixed_atoms()
        reference = None if fixed else self.ReadFrame(frame=0)
        nold = self.frames
        nnew = nold + (nold - 1) * ninsert
        xyz = self.ReadFrame(frame=nold - 1)
        if not fixed:
            xyz = superimpose(xyz, reference)
        inew = nnew
        for n in range(nold - 2, -1, -1):
            start = self.ReadFrame(frame=n)
            if not fixed:
                start = superimpose(start, reference)
            step = (start - xyz) / float(ninsert + 1)
            inew -= 1
            self.WriteFrame(xyz, frame=inew)
            for _ in range(ninsert):
                inew -= 1
                xyz = xyz + step
                self.WriteFrame(xyz, frame=inew)
            xyz = start
        self.frames = nnew

    @classmethod
    def LinearlyInterpolate(cls, path, system, npoints, point0, pointn):
        """A new trajectory of npoints (at least 2) structures from point0 to pointn (SystemGeometryTrajectory.py:
        120-143); without fixed atoms pointn is first superimposed on point0."""
        npoints = max(int(npoints), 2)
        self = cls(path, system, mode="w")
        p0 = np.asarray(point0, dtype=np.float64).reshape(-1, 3)
        pn = np.asarray(pointn, dtype=np.float64).reshape(-1, 3)
        if not self._has_fixed_atoms():
            pn = superimpose(pn, p0)
        step = (pn - p0) / float(npoints - 1)
        self.WriteFrame(p0)
        xyz = p0.copy()
        for _ in range(npoints - 1):
            xyz = xyz + step
            self.WriteFrame(xyz)
        return self

    def Superimpose(self, reference3=None, weights=None):
        """Superimpose every frame on reference3 (frame 0 by default), rewriting the frames; returns the RMS
        deviations before and after per frame (SystemGeometryTrajectory.py:234-255).  The owner keeps its
        coordinates."""
        saved = np.array(self.owner.coordinates3, dtype=np.float64)
        ref = self.ReadFrame(frame=0) if reference3 is None else np.asarray(reference3, dtype=np.float64).reshape(-1, 3)
        results = []
        for index in range(self.frames):
            x = self.ReadFrame(frame=index)
            rms0 = rms_deviation(x, ref, weights)
            y = superimpose(x, ref, weights)
            results.append((rms0, rms_deviation(y, ref, weights)))
            self.WriteFrame(y, frame=index)
        self.owner.coordinates3 = saved
        return results
