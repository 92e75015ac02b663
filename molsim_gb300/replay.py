"""Input and output files of the compiled ABI caller `mg_replay`
(molsim_gb300/harness/mg_replay.cpp).

Both are sequences of tagged arrays: a 16-byte NUL-padded name, a type byte
('i' int32, 'd' float64), an int64 count and the little-endian values.
`write_input` stores a System's mg_params fields, its positions and the run;
`read_output` returns the arrays the harness wrote; `run` does both around
one harness call.
"""
import os
import struct
import subprocess

import numpy as np

from . import abi, units

HARNESS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mg_replay")
RUN_KINDS = {"velver": 0, "bdstep": 1, "mc": 2}

__all__ = ["HARNESS", "write_input", "read_output", "run"]


def _put(f, name, arr):
    a = np.asarray(arr)
    if a.dtype.kind in "iub":
        t, a = b"i", np.ascontiguousarray(a, dtype="<i4")
    else:
        t, a = b"d", np.ascontiguousarray(a, dtype="<f8")
    nm = name.encode()
    if len(nm) > 16:
        raise ValueError(f"array name {name!r} longer than 16 bytes")
    f.write(nm.ljust(16, b"\0") + t + struct.pack("<q", a.size) + a.tobytes())


def write_input(path, system, form, kind, nstep, **run):
    """The system (table built), form (abi.MG_FP64/MG_MIXED) and the run:
    kind 'velver' (tstep, massip, rod, rodd), 'bdstep' (fac1, fac2, iseed)
    or 'mc' (iseed, dtran; beta from the system's temperature)."""
    s = system
    p, keep = s.params(form)
    with open(path, "wb") as f:
        for name in ("iptpn", "iptpt", "az", "ubuf", "iubuflow", "r2umin", "r2atat"):
            _put(f, name, keep[name])
        ints = dict(np=p.np, npt=p.npt, nptpt=p.nptpt, txintlist=p.txintlist, mode=p.mode, form=p.form,
                    maxnneigh=p.maxnneigh, ewald=p.ewald, ncut=p.ncut, ncutregion_cube=p.ncutregion_cube,
                    order=p.order, nmesh=p.nmesh, lsurf=p.lsurf)
        for k, v in ints.items():
            _put(f, k, np.array([v], dtype=np.int32))
        reals = dict(rcut=p.rcut, drnlist=p.drnlist, ualpha=p.ualpha, epsi_four_pi=p.epsi_four_pi,
                     force_fac=p.force_fac)
        for k, v in reals.items():
            _put(f, k, np.array([v], dtype=np.float64))
        _put(f, "boxlen", np.asarray(s.boxlen, dtype=np.float64))
        for name in ("bond_ip", "bond_jp", "bond_k", "bond_eq", "bond_p",
                     "angle_jm", "angle_ip", "angle_jp", "angle_k", "angle_eq", "angle_p"):
            if name in keep:
                _put(f, name, keep[name])
        _put(f, "ro", s.ro_flat())
        _put(f, "run_kind", np.array([RUN_KINDS[kind]], dtype=np.int32))
        _put(f, "nstep", np.array([nstep], dtype=np.int32))
        if kind == "mc":
            run.setdefault("beta", units.sclene / (units.GasConstant * s.temp * units.scltem))
        for k, v in run.items():
            a = np.atleast_1d(np.asarray(v))
            if k == "iseed":
                a = a.astype(np.int32)
            _put(f, k, a)


def read_output(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        name = data[pos:pos + 16].rstrip(b"\0").decode()
        t = data[pos + 16:pos + 17]
        (n,) = struct.unpack_from("<q", data, pos + 17)
        pos += 25
        dt, sz = ("<i4", 4) if t == b"i" else ("<f8", 8)
        out[name] = np.frombuffer(data, dtype=dt, count=n, offset=pos).copy()
        pos += n * sz
    return out


def run(workdir, system, form, kind, nstep, **kw):
    """Write the input, run the harness, return its output arrays."""
    if not os.path.exists(HARNESS):
        raise RuntimeError(f"{HARNESS} is missing; build it with molsim_gb300.build()")
    fin, fout = os.path.join(workdir, "replay.in"), os.path.join(workdir, "replay.out")
    write_input(fin, system, form, kind, nstep, **kw)
    r = subprocess.run([HARNESS, fin, fout], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"mg_replay failed ({r.returncode}): {r.stderr.strip()}")
    return read_output(fout)
