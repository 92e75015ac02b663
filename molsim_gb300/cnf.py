"""The reference's configuration file (`<project>.cnf`), read and written.

IOCnf (molsim.F90:840-965) keeps the configuration in a Fortran unformatted
sequential file: each record is framed by its length in bytes (a 4-byte
little-endian integer before and after it, gfortran's default).  The
records IOCnf writes (`str == 'write'`):

  1. istep1 (int32), iseed (int32), am (real64), ix (int32), iy (int32),
     boxlen(3) (real64)                                   -- the generator state
  2. np (int32), iaux (int32), raux (real64), raux (real64), laux, laux
     (logical, 4 bytes)
  3. (ro(1:3,ip), qua(0:3,ip), ip = 1, np)  (real64)     -- positions, orientations
  4. with crosslinks: nbondcl(1:np), bondcl(1:maxvalnbondcl,1:np) (int32)
  5. with weak charges: laz(1:np) (logical)
  6. MD: (rod(1:3,ip), quad(0:3,ip), ip = 1, np) (real64) -- velocities

`read_cnf` returns the fields of records 1-3 and the MD velocities when a
record of the same size follows; other records are kept raw.  `write_cnf`
writes records 1-3 (and 6 with velocities) in that layout.
"""
import struct

import numpy as np

__all__ = ["read_records", "write_records", "read_cnf", "write_cnf"]


def read_records(path):
    """The payloads of a Fortran unformatted sequential file."""
    with open(path, "rb") as f:
        data = f.read()
    recs, pos = [], 0
    while pos < len(data):
        if pos + 4 > len(data):
            raise ValueError(f"{path}: truncated record marker at byte {pos}")
        (n,) = struct.unpack_from("<i", data, pos)
        end = pos + 4 + n
        if n < 0 or end + 4 > len(data):
            raise ValueError(f"{path}: bad record length {n} at byte {pos}")
        (n2,) = struct.unpack_from("<i", data, end)
        if n2 != n:
            raise ValueError(f"{path}: record markers {n} and {n2} differ at byte {pos}")
        recs.append(data[pos + 4:end])
        pos = end + 4
    return recs


def write_records(path, recs):
    with open(path, "wb") as f:
        for r in recs:
            f.write(struct.pack("<i", len(r)))
            f.write(r)
            f.write(struct.pack("<i", len(r)))


_HEAD = struct.Struct("<iidii3d")        # istep1, iseed, am, ix, iy, boxlen(3)
_COUNTS = struct.Struct("<iiddii")       # np, iaux, raux, raux, laux, laux


def read_cnf(path):
    """Configuration of a .cnf file written by IOCnf('write'):
    dict(istep, iseed, am, ix, iy, boxlen (3,), np, ro (np, 3), qua (np, 4),
    rod and quad (np, 3) / (np, 4) or None, extra: the other raw records)."""
    recs = read_records(path)
    if len(recs) < 3:
        raise ValueError(f"{path}: {len(recs)} records, IOCnf writes at least 3")
    if len(recs[0]) != _HEAD.size:
        raise ValueError(f"{path}: first record has {len(recs[0])} bytes, not {_HEAD.size}")
    istep, iseed, am, ix, iy, bx, by, bz = _HEAD.unpack(recs[0])
    if len(recs[1]) != _COUNTS.size:
        raise ValueError(f"{path}: second record has {len(recs[1])} bytes, not {_COUNTS.size}")
    npart = _COUNTS.unpack(recs[1])[0]
    if len(recs[2]) != 56 * npart:
        raise ValueError(f"{path}: position record has {len(recs[2])} bytes for np = {npart}")
    a = np.frombuffer(recs[2], dtype="<f8").reshape(npart, 7)
    out = dict(istep=istep, iseed=iseed, am=am, ix=ix, iy=iy, boxlen=np.array([bx, by, bz]), np=npart,
               ro=a[:, :3].copy(), qua=a[:, 3:].copy(), rod=None, quad=None, extra=[])
    rest = recs[3:]
    if rest and len(rest[-1]) == 56 * npart:   # MD velocities are the last record
        v = np.frombuffer(rest[-1], dtype="<f8").reshape(npart, 7)
        out["rod"], out["quad"] = v[:, :3].copy(), v[:, 3:].copy()
        rest = rest[:-1]
    out["extra"] = rest
    return out


def write_cnf(path, ro, boxlen, istep=0, iseed=1, am=0.0, ix=-1, iy=-1, qua=None, rod=None, quad=None):
    """Write a .cnf in IOCnf's layout (records 1-3, and 6 with velocities).
    Monoatomic particles carry the unit quaternion (1, 0, 0, 0)."""
    ro = np.asarray(ro, dtype=np.float64).reshape(-1, 3)
    n = ro.shape[0]
    if qua is None:
        qua = np.zeros((n, 4))
        qua[:, 0] = 1.0
    bx, by, bz = (float(x) for x in boxlen)
    recs = [_HEAD.pack(istep, iseed, am, ix, iy, bx, by, bz),
            _COUNTS.pack(n, 0, 0.0, 0.0, 0, 0),
            np.ascontiguousarray(np.hstack([ro, np.asarray(qua, dtype=np.float64)]), dtype="<f8").tobytes()]
    if rod is not None:
        if quad is None:
            quad = np.zeros((n, 4))
        recs.append(np.ascontiguousarray(np.hstack([np.asarray(rod, dtype=np.float64).reshape(-1, 3),
                                                    np.asarray(quad, dtype=np.float64)]), dtype="<f8").tobytes())
    write_records(path, recs)
