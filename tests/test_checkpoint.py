"""Restart files in the reference's format (checkpoint.py, B/saveload.f90).

CPU tests check the Fortran record framing (including split subrecords),
the per-rank pencils, the reference's file names and the particle files'
local arrays.  The GPU test saves a running box, restarts a fresh box and the
CPU oracle from the same files the way the reference restarts
(B/main.f90:124-134), and holds the two restarted runs to the FP64 contract.
"""

import struct

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import checkpoint as ck


def test_record_framing(tmp_path):
    p = tmp_path / "r.bin"
    a = np.arange(6, dtype=np.int32).reshape(2, 3)
    ck.write_records(p, [b"abc", a, np.array([1.5, -2.0])])
    raw = p.read_bytes()
    # marker, data, marker; the array in Fortran (column-major) order
    assert raw[:11] == struct.pack("<i", 3) + b"abc" + struct.pack("<i", 3)
    assert raw[11:15] == struct.pack("<i", 24)
    assert np.array_equal(np.frombuffer(raw[15:39], dtype="<i4"), a.ravel(order="F"))
    recs = ck.read_records(p)
    assert recs[0] == b"abc"
    assert np.array_equal(np.frombuffer(recs[2], dtype="<f8"), [1.5, -2.0])


def test_subrecords(tmp_path):
    p = tmp_path / "s.bin"
    data = bytes(range(40))
    ck.write_records(p, [data, b"xy"], max_subrecord=16)
    raw = p.read_bytes()
    marks = []
    pos = 0
    for n in (16, 16, 8, 2):
        head = struct.unpack("<i", raw[pos:pos + 4])[0]
        tail = struct.unpack("<i", raw[pos + 4 + n:pos + 8 + n])[0]
        marks.append((head, tail))
        pos += 8 + n
    assert marks == [(-16, 16), (-16, -16), (8, -8), (2, 2)]
    assert ck.read_records(p) == [data, b"xy"]


def test_names_follow_the_reference():
    assert ck.flow_name(2000, 7) == "endrunflow2D8x8S1.002000.007"
    assert ck.force_name(15) == "force.000015"
    assert ck.part_name(123456, 63) == "endrunpart2D.123456.063"
    # the leading place is not bounded: char(12 + 48) = '<'
    assert ck.force_name(1234567)[6] == "<"


def test_flow_pencils_roundtrip(tmp_path):
    rng = np.random.default_rng(1)
    f = rng.standard_normal((19, 6, 8, 4))
    ck.write_flow(tmp_path, 40, f, nprocy=4, nprocz=2, nsteps=100, istat=3)
    assert len(list(tmp_path.iterdir())) == 8
    # rank 5 = (indy 1, indz 1): y 2..3, z 2..3
    recs = ck.read_records(tmp_path / ck.flow_name(40, 5))
    part = np.frombuffer(recs[1], dtype="<f8").reshape((19, 6, 2, 2), order="F")
    assert np.array_equal(part, f[:, :, 2:4, 2:4])
    head, g = ck.read_flow(tmp_path, 40, 6, 8, 4, 4, 2)
    assert head == (100, 3, 0)
    assert np.array_equal(g, f)


def test_forcing_roundtrip(tmp_path):
    ivf = np.arange(32, dtype=np.int32) * 7919
    b = np.linspace(-1, 1, 450)
    ck.write_forcing(tmp_path, 9, 232300, ivf, 123, b)
    iseedf, ivf2, iyf, b2 = ck.read_forcing(tmp_path, 9)
    assert (iseedf, iyf) == (232300, 123)
    assert np.array_equal(ivf2, ivf) and np.array_equal(b2, b)


def test_particles_roundtrip(tmp_path):
    rng = np.random.default_rng(2)
    nx, ny, nz, npart = 8, 16, 12, 12
    st = {"ypglb": rng.uniform(0, 1, (npart, 3)) * [nx, ny, nz]}
    for k in ("wp", "omgp") + ck.LOCAL:
        st[k] = rng.standard_normal((npart, 3))
    isn = rng.integers(-1, npart, (nx, ny, nz)).astype(np.int32)
    ck.write_particles(tmp_path, 5, st, isn, nprocy=2, nprocz=2)
    back, isn2 = ck.read_particles(tmp_path, 5, npart, nx, ny, nz, 2, 2)
    for k in st:
        assert np.array_equal(back[k], st[k]), k
    assert np.array_equal(isn2, isn)
    # rank 3 holds the particles with y >= 8 and z >= 6, 1-based ids
    recs = ck.read_records(tmp_path / ck.part_name(5, 3))
    nps = struct.unpack("<i", recs[0][:4])[0]
    ids = np.frombuffer(recs[0][4:], dtype="<i4")[:nps]
    mine = [p + 1 for p in range(npart) if st["ypglb"][p, 1] >= 8 and st["ypglb"][p, 2] >= 6]
    assert list(ids) == mine
    assert ck.npart_in_files(tmp_path, 5) == npart


def test_particles_beyond_msize_rejected(tmp_path):
    st = {"ypglb": np.array([[1.0, 1.0, 1.0]] * 4)}
    for k in ("wp", "omgp") + ck.LOCAL:
        st[k] = np.zeros((4, 3))
    # msize = int(5 * 4 / 4) = 5 per rank; all four in rank 0 fits, then
    # with 16 ranks msize = 1 does not
    ck.write_particles(tmp_path, 1, st, np.full((4, 4, 4), -1, np.int32), 2, 2)
    with pytest.raises(ValueError):
        ck.write_particles(tmp_path, 1, st, np.full((4, 4, 4), -1, np.int32), 4, 4)


@pytest.mark.gpu
def test_restart_matches_oracle_restart(require_gpu, oracle_mod, tmp_path):
    from conftest import relerr
    from test_gpu_parity import TOL64, make_pair
    from multiphase_flow_codes_gb300 import _capi as capi
    from multiphase_flow_codes_gb300.engine import LBMBox

    shape = (32, 32, 32)
    _, a = make_pair(oracle_mod, shape=shape, npart=4, rad=4.0, rhopart=2.5)
    a.step(6)
    ck.save(a, tmp_path, 6, nprocy=2, nprocz=2, nsteps=6)
    cfg = capi.config_init(capi.LBM_PRESET_BOX, *shape, 4, 4.0, 2.5)

    b = LBMBox(cfg)
    ck.load(b, tmp_path, 6, 2, 2)
    assert b.npart == 4

    o = oracle_mod.OracleBox(cfg)
    _, f = ck.read_flow(tmp_path, 6, *shape, 2, 2)
    o.f[...] = np.transpose(f, (0, 3, 2, 1))
    iseedf, ivf, iyf, bb = ck.read_forcing(tmp_path, 6)
    o.set_forcing_state(iseedf, iyf, ivf, bb)
    st, _ = ck.read_particles(tmp_path, 6, 4, *shape, 2, 2)
    o.restore_particles(st)
    o.macrovar()

    # the restarted state itself: populations and particles as saved
    assert np.array_equal(b.get_f(), a.get_f())
    pa, pb = a.get_particle_state(), b.get_particle_state()
    for k in ("ypglb", "wp", "omgp") + ck.LOCAL:
        assert np.array_equal(pb[k], pa[k]), k
    assert pb["first_move"] == 0
    assert np.array_equal(b.get_flags()[1], a.get_flags()[1])
    for _ in range(6):
        o.step(1)
        b.step(1)
    assert relerr(b.get_f(), o.f) <= TOL64
    assert relerr(b.get_particles()["ypglb"], np.asarray(o.ypglb)[:4]) <= TOL64
