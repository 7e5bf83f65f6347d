"""Restart files in the reference's own format (B/saveload.f90).

A GPU run can resume from a reference run's restart files and hand its state
back to the reference.  The reference writes Fortran unformatted sequential
files, one per MPI rank of its pencil decomposition (B/para.f90:184-198:
rank myid = indz * nprocY + indy holds y in [indy*ly, (indy+1)*ly) and z in
[indz*lz, (indz+1)*lz), ly = ny/nprocY, lz = nz/nprocZ, all x):

  endrunflow2D8x8S1.<istep>.<myid>   savecntdflow / loadcntdflow
                                     (saveload.f90:180-211, 276-308)
      record 1: nsteps, istat, imovie           integer*4
      record 2: f(0:18, lx, ly, lz)             real*8, the rank's pencil
  force.<istep>                      input_outputf (saveload.f90:212-274)
      iseedf | ivf(32) | iyf | b1r, b2r, b3r (each (6,5,5) real*8)
  endrunpart2D.<istep>.<myid>        savecntdpart / loadcntdpart
                                     (saveload.f90:582-665)
      nps, ipglb(msize) | ibnodes0, isnodes0 (lx, ly, lz) |
      yp, thetap (3, msize) | forcepp, torqpp | dwdt, domgdt |
      rank 0 only: ypglb, wp, omgp (3, npart)

with msize = int(5 npart / nproc) (para.f90:248) and 1-based particle ids.
Step and rank numbers are spelled digit by digit as the reference does
(char(d + 48), six digits for the step, three for the rank).

Each record is framed by 4-byte little-endian length markers, as gfortran
and ifort write them; a record longer than 2^31 - 9 bytes is split into
subrecords whose head marker is negative while the record continues (and
whose tail marker is negative for every subrecord after the first).  The
reference is built with 8-byte reals (it passes `real` arrays as
MPI_REAL8).  Populations are the deviations f - w rho0 in both codes.

`save` and `load` move an LBMBox to and from these files.  `load` follows
the reference's restart (B/main.f90:124-134): populations, forcing state,
particles with their flags and links rebuilt from the positions, then
macrovar with no force (the force arrays of a fresh reference process are
not yet computed); the first step's FORCING then draws from the restored
generator.
"""

from __future__ import annotations

import os
import struct

import numpy as np

MAX_SUBRECORD = 2147483639  # gfortran's largest subrecord (2^31 - 9 bytes)


# ---- Fortran unformatted sequential records -------------------------------
def write_records(path, records, max_subrecord: int = MAX_SUBRECORD):
    """Write each item of `records` (bytes or arrays, written in Fortran
    order) as one record."""
    with open(path, "wb") as fh:
        for rec in records:
            data = rec if isinstance(rec, (bytes, bytearray)) else _fortran_bytes(rec)
            n = len(data)
            if n <= max_subrecord:
                fh.write(struct.pack("<i", n))
                fh.write(data)
                fh.write(struct.pack("<i", n))
                continue
            pos, first = 0, True
            while pos < n:
                m = min(max_subrecord, n - pos)
                last = pos + m >= n
                fh.write(struct.pack("<i", m if last else -m))
                fh.write(data[pos:pos + m])
                fh.write(struct.pack("<i", m if first else -m))
                pos += m
                first = False


def read_records(path) -> list:
    """Every record of the file as bytes (subrecords joined)."""
    out = []
    with open(path, "rb") as fh:
        while True:
            head = fh.read(4)
            if not head:
                break
            if len(head) < 4:
                raise ValueError(f"{path}: truncated record marker")
            parts = []
            while True:
                (m,) = struct.unpack("<i", head)
                n = abs(m)
                data = fh.read(n)
                tail = fh.read(4)
                if len(data) < n or len(tail) < 4:
                    raise ValueError(f"{path}: truncated record")
                if abs(struct.unpack("<i", tail)[0]) != n:
                    raise ValueError(f"{path}: record markers disagree")
                parts.append(data)
                if m >= 0:
                    break
                head = fh.read(4)
                if len(head) < 4:
                    raise ValueError(f"{path}: missing continuation subrecord")
            out.append(b"".join(parts))
    return out


def _fortran_bytes(a) -> bytes:
    a = np.asarray(a)
    return np.asfortranarray(a).tobytes(order="F")


def _split(data: bytes, specs) -> list:
    """Cut one record into arrays: specs = [(dtype, shape), ...] in order."""
    out, pos = [], 0
    for dt, shape in specs:
        dt = np.dtype(dt).newbyteorder("<")
        n = int(np.prod(shape)) * dt.itemsize
        if pos + n > len(data):
            raise ValueError("record shorter than expected")
        out.append(np.frombuffer(data[pos:pos + n], dtype=dt).reshape(shape, order="F").copy())
        pos += n
    if pos != len(data):
        raise ValueError(f"record of {len(data)} bytes, expected {pos}")
    return out


# ---- names and decomposition ---------------------------------------------
def _digits(v: int, n: int) -> str:
    """char(d + 48) for the n decimal places of v, the leading one unbounded
    (saveload.f90:190-201)."""
    out = []
    for k in range(n - 1, -1, -1):
        d = v // 10 ** k if k == n - 1 else (v % 10 ** (k + 1)) // 10 ** k
        out.append(chr(d + 48))
    return "".join(out)


def flow_name(istep: int, myid: int) -> str:
    return f"endrunflow2D8x8S1.{_digits(istep, 6)}.{_digits(myid, 3)}"


def force_name(istep: int) -> str:
    return f"force.{_digits(istep, 6)}"


def part_name(istep: int, myid: int) -> str:
    return f"endrunpart2D.{_digits(istep, 6)}.{_digits(myid, 3)}"


def pencils(ny: int, nz: int, nprocy: int, nprocz: int):
    """(myid, y0, y1, z0, z1) of every rank (para.f90:184-198)."""
    if ny % nprocy or nz % nprocz:
        raise ValueError("ny and nz must be multiples of nprocY and nprocZ")
    ly, lz = ny // nprocy, nz // nprocz
    for myid in range(nprocy * nprocz):
        indy, indz = myid % nprocy, myid // nprocy
        yield myid, indy * ly, (indy + 1) * ly, indz * lz, (indz + 1) * lz


def msize(npart: int, nproc: int) -> int:
    """para.f90:248"""
    return int(5.0 * float(npart) / float(nproc))


# ---- flow ------------------------------------------------------------------
def write_flow(dirpath, istep: int, f, nprocy: int, nprocz: int, nsteps: int = 0,
               istat: int = 0, imovie: int = 0):
    """f: (19, nx, ny, nz) in the reference's index order."""
    f = np.asarray(f, dtype=np.float64)
    _, nx, ny, nz = f.shape
    for myid, y0, y1, z0, z1 in pencils(ny, nz, nprocy, nprocz):
        head = struct.pack("<3i", nsteps, istat, imovie)
        write_records(os.path.join(dirpath, flow_name(istep, myid)), [head, f[:, :, y0:y1, z0:z1]])


def read_flow(dirpath, istep: int, nx: int, ny: int, nz: int, nprocy: int, nprocz: int):
    """((nsteps, istat, imovie) of rank 0, f (19, nx, ny, nz) Fortran order)."""
    f = np.zeros((19, nx, ny, nz), dtype=np.float64, order="F")
    head0 = None
    for myid, y0, y1, z0, z1 in pencils(ny, nz, nprocy, nprocz):
        recs = read_records(os.path.join(dirpath, flow_name(istep, myid)))
        if len(recs) != 2:
            raise ValueError(f"{flow_name(istep, myid)}: {len(recs)} records, expected 2")
        (head,) = _split(recs[0], [(np.int32, (3,))])
        (part,) = _split(recs[1], [(np.float64, (19, nx, y1 - y0, z1 - z0))])
        f[:, :, y0:y1, z0:z1] = part
        if head0 is None:
            head0 = tuple(int(v) for v in head)
    return head0, f


# ---- forcing ---------------------------------------------------------------
def write_forcing(dirpath, istep: int, iseedf: int, ivf, iyf: int, b):
    b = np.asarray(b, dtype=np.float64).reshape(450)
    write_records(os.path.join(dirpath, force_name(istep)),
                  [struct.pack("<i", iseedf), np.asarray(ivf, dtype=np.int32).reshape(32),
                   struct.pack("<i", iyf), b])


def read_forcing(dirpath, istep: int):
    """(iseedf, ivf[32], iyf, b[450] = b1r, b2r, b3r)"""
    recs = read_records(os.path.join(dirpath, force_name(istep)))
    if len(recs) != 4:
        raise ValueError(f"{force_name(istep)}: {len(recs)} records, expected 4")
    (iseedf,) = _split(recs[0], [(np.int32, (1,))])
    (ivf,) = _split(recs[1], [(np.int32, (32,))])
    (iyf,) = _split(recs[2], [(np.int32, (1,))])
    (b,) = _split(recs[3], [(np.float64, (450,))])
    return int(iseedf[0]), ivf, int(iyf[0]), b


# ---- particles -------------------------------------------------------------
LOCAL = ("thetap", "forcepp", "torqpp", "dwdt", "domgdt")


def write_particles(dirpath, istep: int, state: dict, isnodes, nprocy: int, nprocz: int):
    """state: (npart, 3) arrays by var_inc name (ypglb, wp, omgp and the
    LOCAL ones); isnodes: (nx, ny, nz) particle ids, 0-based, -1 fluid."""
    y = np.asarray(state["ypglb"], dtype=np.float64).reshape(-1, 3)
    npart = y.shape[0]
    isn = np.asarray(isnodes, dtype=np.int32)
    nx, ny, nz = isn.shape
    nproc = nprocy * nprocz
    ms = msize(npart, nproc)
    for myid, y0, y1, z0, z1 in pencils(ny, nz, nprocy, nprocz):
        # beads_redistribute's ownership test (partlib.f90:2445-2480)
        mine = [p for p in range(npart)
                if float(y0) <= y[p, 1] < float(y1) and float(z0) <= y[p, 2] < float(z1)]
        if len(mine) > ms:
            raise ValueError(f"rank {myid} holds {len(mine)} particles > msize {ms}")
        ipglb = np.zeros(ms, dtype=np.int32)
        ipglb[:len(mine)] = np.array(mine, dtype=np.int32) + 1

        def local(name):
            a = np.zeros((3, ms), dtype=np.float64, order="F")
            if mine:
                a[:, :len(mine)] = np.asarray(state[name], dtype=np.float64).reshape(-1, 3)[mine].T
            return a

        loc = isn[:, y0:y1, z0:z1]
        ib0 = np.where(loc >= 0, 1, -1).astype(np.int32)
        is0 = np.where(loc >= 0, loc + 1, -1).astype(np.int32)
        recs = [struct.pack("<i", len(mine)) + _fortran_bytes(ipglb),
                _fortran_bytes(ib0) + _fortran_bytes(is0),
                _fortran_bytes(local("ypglb")) + _fortran_bytes(local("thetap")),
                _fortran_bytes(local("forcepp")) + _fortran_bytes(local("torqpp")),
                _fortran_bytes(local("dwdt")) + _fortran_bytes(local("domgdt"))]
        if myid == 0:
            recs.append(b"".join(_fortran_bytes(np.asarray(state[k], dtype=np.float64)
                                                .reshape(-1, 3).T) for k in ("ypglb", "wp", "omgp")))
        write_records(os.path.join(dirpath, part_name(istep, myid)), recs)


def read_particles(dirpath, istep: int, npart: int, nx: int, ny: int, nz: int, nprocy: int,
                   nprocz: int):
    """(state with (npart, 3) arrays ypglb, wp, omgp and LOCAL, isnodes0
    (nx, ny, nz) 0-based with -1 fluid)."""
    nproc = nprocy * nprocz
    ms = msize(npart, nproc)
    state = {k: np.zeros((npart, 3)) for k in ("ypglb", "wp", "omgp") + LOCAL}
    isn = np.full((nx, ny, nz), -1, dtype=np.int32, order="F")
    for myid, y0, y1, z0, z1 in pencils(ny, nz, nprocy, nprocz):
        recs = read_records(os.path.join(dirpath, part_name(istep, myid)))
        if len(recs) != (6 if myid == 0 else 5):
            raise ValueError(f"{part_name(istep, myid)}: {len(recs)} records")
        nps, ipglb = _split(recs[0], [(np.int32, (1,)), (np.int32, (ms,))])
        nps = int(nps[0])
        shp = (nx, y1 - y0, z1 - z0)
        _, is0 = _split(recs[1], [(np.int32, shp), (np.int32, shp)])
        isn[:, y0:y1, z0:z1] = np.where(is0 > 0, is0 - 1, -1)
        v = (np.float64, (3, ms))
        yp, thetap = _split(recs[2], [v, v])
        forcepp, torqpp = _split(recs[3], [v, v])
        dwdt, domgdt = _split(recs[4], [v, v])
        ids = ipglb[:nps] - 1
        for name, arr in (("thetap", thetap), ("forcepp", forcepp), ("torqpp", torqpp),
                          ("dwdt", dwdt), ("domgdt", domgdt)):
            state[name][ids] = arr[:, :nps].T
        if myid == 0:
            g = (np.float64, (3, npart))
            yg, wp, om = _split(recs[5], [g, g, g])
            state["ypglb"][:] = yg.T
            state["wp"][:] = wp.T
            state["omgp"][:] = om.T
    return state, isn


# ---- an LBMBox to and from the files ---------------------------------------
def save(box, dirpath, istep: int, nprocy: int, nprocz: int, nsteps: int = 0):
    """Write the box's populations, forcing state and particles (FP64
    boxes: the files hold real*8)."""
    os.makedirs(dirpath, exist_ok=True)
    write_flow(dirpath, istep, box.get_f_fortran(), nprocy, nprocz, nsteps=nsteps)
    try:
        iseedf, iyf, ivf, b = box.get_forcing_state()
    except Exception:
        iseedf = None
    if iseedf is not None:
        write_forcing(dirpath, istep, iseedf, ivf, iyf, b)
    if box.npart > 0:
        st = box.get_particle_state()
        _, isn = box.get_flags()  # (nz, ny, nx)
        write_particles(dirpath, istep, st, np.transpose(isn, (2, 1, 0)), nprocy, nprocz)


def npart_in_files(dirpath, istep: int) -> int:
    """The particle count of a checkpoint (rank 0's last record), 0 if none."""
    path = os.path.join(dirpath, part_name(istep, 0))
    if not os.path.exists(path):
        return 0
    return len(read_records(path)[-1]) // (3 * 3 * 8)


def load(box, dirpath, istep: int, nprocy: int, nprocz: int, npart: int | None = None):
    """The reference's restart (B/main.f90:124-134) into a fresh box."""
    if npart is None:
        npart = npart_in_files(dirpath, istep)
    _, f = read_flow(dirpath, istep, box.nx, box.ny, box.nz, nprocy, nprocz)
    box.set_f_fortran(f)
    if os.path.exists(os.path.join(dirpath, force_name(istep))):
        iseedf, ivf, iyf, b = read_forcing(dirpath, istep)
        box.set_forcing_state(iseedf, iyf, ivf, b)
    if npart > 0:
        st, _ = read_particles(dirpath, istep, npart, box.nx, box.ny, box.nz, nprocy, nprocz)
        box.set_particle_state(st, first_move=0)
    box.macrovar()
