"""State persistence with the datasets of the reference's simpleModelDatabase
(src/databases/simpleModelDatabase.cpp:9-158), in the flat binary layout of include/curvedSpaceSimDatabase.hpp:

    header (24 bytes): b"CSSGDB01", int32 N, int32 flags (1 velocity, 2 force, 4 type), int64 reserved
    record:            float64 time, float64 R3position[3N], float64 barycentricPosition[3N], int32 faceIndex[N],
                       [float64 velocity[3N]], [float64 force[3N]], [int32 type[N]]

All values little-endian; records have a fixed size, so readState(rec) seeks directly.
"""
from __future__ import annotations

import os

import numpy as np

MAGIC = b"CSSGDB01"
READONLY, READWRITE, REPLACE = "readonly", "readwrite", "replace"


class SimpleModelDatabase:
    def __init__(self, n: int, filename: str, mode: str = REPLACE, save_velocities=False, save_types=False,
                 save_forces=False):
        self.N = int(n)
        self.filename = filename
        self.mode = mode
        self.velocity, self.type, self.force = bool(save_velocities), bool(save_types), bool(save_forces)
        if mode == REPLACE or (mode == READWRITE and not os.path.exists(filename)):
            self._write_header()
        else:
            with open(filename, "rb") as fh:
                head = fh.read(24)
            if len(head) != 24 or head[:8] != MAGIC:
                raise ValueError(f"{filename} is not a curvedSpaceSim database")
            hn, flags = np.frombuffer(head[8:16], dtype="<i4")
            if hn != self.N:
                raise ValueError(f"{filename} holds {hn} particles, not {self.N}")
            self.velocity, self.force, self.type = bool(flags & 1), bool(flags & 2), bool(flags & 4)

    def _write_header(self):
        flags = (1 if self.velocity else 0) | (2 if self.force else 0) | (4 if self.type else 0)
        with open(self.filename, "wb") as fh:
            fh.write(MAGIC + np.array([self.N, flags], dtype="<i4").tobytes() + np.zeros(1, "<i8").tobytes())

    @property
    def record_bytes(self) -> int:
        n = self.N
        b = 8 + 48 * n + 4 * n
        if self.velocity:
            b += 24 * n
        if self.force:
            b += 24 * n
        if self.type:
            b += 4 * n
        return b

    def current_number_of_records(self) -> int:
        size = os.path.getsize(self.filename)
        return max(0, (size - 24) // self.record_bytes)

    def write_state(self, time, r3, bary, face, velocity=None, force=None, types=None):
        if self.mode == READONLY:
            raise PermissionError("database opened read-only")
        n = self.N
        parts = [np.array([time], "<f8").tobytes(), np.asarray(r3, "<f8").reshape(3 * n).tobytes(),
                 np.asarray(bary, "<f8").reshape(3 * n).tobytes(), np.asarray(face, "<i4").reshape(n).tobytes()]
        if self.velocity:
            parts.append(np.asarray(velocity, "<f8").reshape(3 * n).tobytes())
        if self.force:
            parts.append(np.asarray(force, "<f8").reshape(3 * n).tobytes())
        if self.type:
            parts.append(np.asarray(types if types is not None else np.zeros(n), "<i4").reshape(n).tobytes())
        with open(self.filename, "ab") as fh:
            fh.write(b"".join(parts))

    def read_state(self, rec: int) -> dict:
        if not 0 <= rec < self.current_number_of_records():
            raise IndexError(f"no record {rec}")
        n = self.N
        with open(self.filename, "rb") as fh:
            fh.seek(24 + rec * self.record_bytes)
            raw = fh.read(self.record_bytes)
        out, o = {}, 0

        def take(name, dtype, count, shape):
            nonlocal o
            size = np.dtype(dtype).itemsize * count
            out[name] = np.frombuffer(raw[o:o + size], dtype=dtype).reshape(shape).copy()
            o += size

        take("time", "<f8", 1, ())
        take("R3position", "<f8", 3 * n, (n, 3))
        take("barycentricPosition", "<f8", 3 * n, (n, 3))
        take("faceIndex", "<i4", n, (n,))
        if self.velocity:
            take("velocity", "<f8", 3 * n, (n, 3))
        if self.force:
            take("force", "<f8", 3 * n, (n, 3))
        if self.type:
            take("type", "<i4", n, (n,))
        out["time"] = float(out["time"])
        return out


VV_MAGIC = b"CSSGVV01"


class ValueVectorDatabase:
    """valueVectorDatabase (src/databases/vectorValueDatabase.cpp:4-43): per record one float64 value and a float64
    vector of fixed size, in the flat layout of include/curvedSpaceSimDatabase.hpp:

        header (24 bytes): b"CSSGVV01", int64 vectorSize, int64 reserved
        record:            float64 value, float64 vector[vectorSize]
    """

    def __init__(self, filename: str, vector_size: int, mode: str = READONLY):
        self.filename = filename
        self.size = int(vector_size)
        self.mode = mode
        if mode == REPLACE or (mode == READWRITE and not os.path.exists(filename)):
            with open(filename, "wb") as fh:
                fh.write(VV_MAGIC + np.array([self.size, 0], dtype="<i8").tobytes())
        else:
            with open(filename, "rb") as fh:
                head = fh.read(24)
            if len(head) != 24 or head[:8] != VV_MAGIC or int(np.frombuffer(head[8:16], "<i8")[0]) != self.size:
                raise ValueError(f"{filename} is not a value/vector database of vectors of size {self.size}")

    def current_number_of_records(self) -> int:
        return max(0, (os.path.getsize(self.filename) - 24) // (8 * (1 + self.size)))

    def write_state(self, value: float, vector):
        if self.mode == READONLY:
            raise PermissionError("database opened read-only")
        vec = np.asarray(vector, "<f8").reshape(-1)
        if vec.size < self.size:
            raise ValueError("vector shorter than the record")
        with open(self.filename, "ab") as fh:
            fh.write(np.array([value], "<f8").tobytes() + vec[: self.size].tobytes())

    def read_state(self, rec: int):
        if not 0 <= rec < self.current_number_of_records():
            raise IndexError(f"no record {rec}")
        with open(self.filename, "rb") as fh:
            fh.seek(24 + rec * 8 * (1 + self.size))
            raw = np.frombuffer(fh.read(8 * (1 + self.size)), "<f8")
        return float(raw[0]), raw[1:].copy()


def write_system(db: SimpleModelDatabase, system, mesh_V, mesh_F, time: float):
    """Append the state of an api.System (one record)."""
    from . import meshes as ms
    f, b, v, frc = system.get_state()
    db.write_state(time, ms.bary_to_r3(mesh_V, mesh_F, f, b), b, f, v, frc)


def read_system(db: SimpleModelDatabase, system, rec: int) -> float:
    """Load record `rec` into an api.System (fields the database lacks keep their current values)."""
    r = db.read_state(rec)
    f, b, v, frc = system.get_state()
    system.set_state(r["faceIndex"], r["barycentricPosition"], r.get("velocity", v), r.get("force", frc))
    return r["time"]
