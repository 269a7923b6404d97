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
DCDTrajectoryFileReader reads such files back (fixed atoms take their first-frame positions).  Host-side I/O:
the dynamics driver copies the replica it saves from the device.
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
