"""GPU parity: the CUDA engine (through the C ABI) against the CPU oracle.

Tolerances, as the path's contract states them:
  * integer work (solid flags, link sets, refill events) must match bit for
    bit; link fractions (FP64 data) within 1e-13;
  * FP64 populations, macroscopic fields and particle state within 1e-12
    (max-norm relative) over 10 steps; the hydrodynamic force and torque
    (fHIp, torqp) within 1e-12 relative to the sum of the magnitudes of the
    particle's link terms, because they are sums over hundreds of links that
    cancel to a small fraction of the terms (their rounding scales with the
    terms, whatever the order of summation);
  * FP32-shifted populations within 1e-5 of the FP64 oracle over 10 steps.
"""

import numpy as np
import pytest

from conftest import gpu_links, link_term_scale, oracle_links, relerr

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def make_pair(oracle_mod, preset=capi.LBM_PRESET_BOX, shape=(32, 32, 32), npart=0, rad=4.5,
              rhopart=5.0, urms=0.03, k0=4.0, precision=capi.LBM_PREC_F64, wp=None, omgp=None,
              mrt_type=None):
    from multiphase_flow_codes_gb300.engine import LBMBox
    nx, ny, nz = shape
    cfg = capi.config_init(preset, nx, ny, nz, npart, rad, rhopart)
    if mrt_type is not None:
        cfg.mrt_type = mrt_type
    cfg.precision = precision
    o = oracle_mod.OracleBox(cfg)
    if urms > 0:
        u = inputs.spectral_velocity(nx, k0, urms, ny=ny, nz=nz)
    else:
        u = tuple(np.zeros((nz, ny, nx)) for _ in range(3))
    o.initpop(*u)
    o.macrovar()
    box = LBMBox(cfg)
    box.set_f(o.f.copy())
    box.macrovar()
    if npart:
        chan = preset == capi.LBM_PRESET_CHANNEL
        y = inputs.initpartpos(nx, ny, nz, npart, rad, channel=chan)
        o.release_particles(y, wp, omgp)
        box.release_particles(y, wp, omgp)
    return o, box


def check_links(o, box, tol_alpha=None):
    po, no, qo, ao = oracle_links(o)
    pg, ng, qg, ag = gpu_links(box)
    assert len(po) == len(pg), (len(po), len(pg))
    assert np.array_equal(po, pg) and np.array_equal(no, ng) and np.array_equal(qo, qg)
    # the link set is integer work (bit-exact); alpha is FP64 data computed
    # from the same root in a better-conditioned form, whose difference from
    # the reference's form is the rounding of the node coordinates (up to n)
    if tol_alpha is None:
        tol_alpha = alpha_tolerance(o)
    assert np.abs(ao - ag).max() <= tol_alpha, np.abs(ao - ag).max()


def alpha_tolerance(o):
    """Link fractions: 16 ulps of the largest node coordinate."""
    return 16.0 * np.finfo(np.float64).eps * max(o.nx, o.ny, o.nz)


def check_force_torque(o, box, tol=TOL64):
    """fHIp and torqp against the oracle, relative to the link-term scale;
    returns the worst errors (scaled, and in the max norm for the record)."""
    links = oracle_links(o)
    n = box.npart
    p = box.get_particles()
    scale = link_term_scale(o, links)[:n, None]
    out = {}
    for k in ("fHIp", "torqp"):
        d = np.abs(p[k] - getattr(o, k)[:n])
        out[k] = float((d / np.maximum(scale, 1e-300)).max())
        out[k + "_maxnorm"] = relerr(p[k], getattr(o, k)[:n])
        assert out[k] <= tol, (k, out)
    return out


def check_flags(o, box):
    ib, isn = box.get_flags()
    assert np.array_equal(ib, o.ibnodes)
    assert np.array_equal(isn, o.isnodes)


def test_fused_periodic_no_particles(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod)
    for s in range(10):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64
    rho, ux, uy, uz = box.get_macro()
    assert relerr(ux, o.ux) <= TOL64 and relerr(uy, o.uy) <= TOL64 and relerr(uz, o.uz) <= TOL64
    fx, fy, fz = box.get_force()
    assert relerr(fx, o.fx) <= TOL64 and relerr(fz, o.fz) <= TOL64


def test_forcing_state_matches(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(16, 16, 16))
    for _ in range(3):
        o.FORCING()
        box.FORCING()
    iseed, iy, iv, b = box.get_forcing_state()
    assert iseed == o.iseedf and iy == o.iyf
    assert np.array_equal(iv, o.ivf)
    bo = np.concatenate([o.b1r, o.b2r, o.b3r])
    assert relerr(b, bo) <= 1e-14


def test_forcing_generator_known_answer(require_gpu, oracle_mod):
    """The device's ranff state after k FORCING calls (450 draws each, drawn
    by jump-ahead) is the minimal-standard sequence from seed 1: after the
    40-step warm-up and 450 k draws, 16807^(40 + 450 k) mod (2^31 - 1)
    (Park & Miller, CACM 1988)."""
    o, box = make_pair(oracle_mod, shape=(16, 16, 16))
    box.set_forcing_state(-1, 0, np.zeros(32, dtype=np.int32), np.zeros(450))
    for k in range(1, 4):
        box.FORCING()
        iseed, _, _, _ = box.get_forcing_state()
        assert iseed == pow(16807, 40 + 450 * k, 2**31 - 1), k
        assert iseed == oracle_mod.ran1_state(1, 450 * k)


def test_unfused_subroutines_match(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(24, 20, 16), npart=2, rad=3.5)
    for s in range(4):
        o.step(1)
        box.step_unfused(1)
        check_flags(o, box)
    assert relerr(box.get_f(), o.f) <= TOL64


def test_links_bit_exact_at_release(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(48, 48, 48), npart=12, rad=4.5)
    check_flags(o, box)
    check_links(o, box)


def test_links_wrapping_particles(require_gpu, oracle_mod):
    """Spheres straddling the periodic faces and corners."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 32, 32, 32, 3, 4.5, 5.0)
    o = oracle_mod.OracleBox(cfg)
    box = LBMBox(cfg)
    y = np.array([[0.3, 31.9, 15.2], [16.1, 0.05, 31.7], [31.99, 16.5, 0.4]])
    o.release_particles(y)
    box.release_particles(y)
    check_flags(o, box)
    check_links(o, box)


def test_particles_box64_geometry_10_steps(require_gpu, oracle_mod):
    """The 64^3, 16-sphere (R = 4.5, density ratio 5) workload, 10 steps."""
    o, box = make_pair(oracle_mod, shape=(64, 64, 64), npart=16, rad=4.5, rhopart=5.0)
    for s in range(10):
        o.step(1)
        box.step(1)
        check_flags(o, box)
        p = box.get_particles()
        assert relerr(p["ypglb"], o.ypglb) <= TOL64
        e = check_force_torque(o, box)
    print(f"\nbox64_p16, 10 steps: {e}")
    assert relerr(box.get_f(), o.f) <= TOL64
    check_links(o, box)


def test_moving_particles_refill(require_gpu, oracle_mod):
    """Spheres launched with translation and spin so that nodes are
    uncovered and refilled every step."""
    rng = np.random.default_rng(7)
    wp = rng.uniform(-0.08, 0.08, (6, 3))
    om = rng.uniform(-0.01, 0.01, (6, 3))
    o, box = make_pair(oracle_mod, shape=(40, 40, 40), npart=6, rad=4.0, rhopart=2.5, wp=wp, omgp=om)
    refilled = 0
    for s in range(10):
        before = o.ibnodes.copy()
        o.step(1)
        box.step(1)
        refilled += int(((before > 0) & (o.ibnodes < 0)).sum())
        check_flags(o, box)
        assert relerr(box.get_f(), o.f) <= TOL64
    assert refilled > 0
    p = box.get_particles()
    assert relerr(p["ypglb"], o.ypglb) <= TOL64
    print(f"\nrefill: omgp {relerr(p['omgp'], o.omgp):.2e} wp {relerr(p['wp'], o.wp):.2e}")
    assert relerr(p["omgp"], o.omgp) <= TOL64
    assert relerr(p["wp"], o.wp) <= TOL64
    check_force_torque(o, box)
    check_links(o, box)


def test_channel_particles(require_gpu, oracle_mod):
    rng = np.random.default_rng(3)
    wp = rng.uniform(-0.05, 0.05, (4, 3))
    o, box = make_pair(oracle_mod, preset=capi.LBM_PRESET_CHANNEL, shape=(30, 36, 28), npart=4,
                       rad=4.0, rhopart=1.0, wp=wp)
    check_links(o, box)
    for s in range(10):
        o.step(1)
        box.step(1)
        check_flags(o, box)
    assert relerr(box.get_f(), o.f) <= TOL64
    p = box.get_particles()
    assert relerr(p["flubp"], o.flubp) <= TOL64


def test_channel_wall_lubrication(require_gpu, oracle_mod):
    """Spheres inside the particle-wall lubrication range of both channel
    walls (centre closer than rad + mingap_w to x = 0 or x = nx,
    3DChannel.../partlib.f90:2317-2356) and a pair inside the
    particle-particle range: the lubrication forces are nonzero and match
    the oracle every step."""
    from multiphase_flow_codes_gb300.engine import LBMBox
    shape = (36, 40, 32)
    cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, *shape, 4, 4.0, 1.0)
    o = oracle_mod.OracleBox(cfg)
    u = tuple(np.zeros((shape[2], shape[1], shape[0])) for _ in range(3))
    o.initpop(*u)
    o.macrovar()
    box = LBMBox(cfg)
    box.set_f(o.f.copy())
    box.macrovar()
    y = np.array([[5.1, 8.3, 7.7],               # 1.1 from the wall x = 0
                  [shape[0] - 5.4, 30.2, 20.6],  # 1.4 from the wall x = nx
                  [18.0, 20.0, 9.0], [18.3, 29.1, 9.4]])  # pair 1.1 apart
    wp = np.array([[-0.01, 0.0, 0.0], [0.01, 0.0, 0.0], [0.0, 0.01, 0.0], [0.0, -0.01, 0.0]])
    o.release_particles(y, wp)
    box.release_particles(y, wp)
    worst = 0.0
    for s in range(10):
        o.step(1)
        box.step(1)
        check_flags(o, box)
        p = box.get_particles()
        if s == 0:  # every sphere starts inside a lubrication range
            assert np.all(np.abs(o.flubp[:4]).max(axis=1) > 0), o.flubp[:4]
        e = relerr(p["flubp"], o.flubp[:4])
        worst = max(worst, e)
        assert e <= TOL64, (s, e)
        assert relerr(p["ypglb"], o.ypglb[:4]) <= TOL64
    print(f"\nwall lubrication: flubp worst {worst:.2e}")
    assert relerr(box.get_f(), o.f) <= TOL64


def test_fp32_shifted_close_to_fp64(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(32, 32, 32), npart=4, rad=4.0, rhopart=2.5,
                       precision=capi.LBM_PREC_F32)
    for s in range(10):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL32
    p = box.get_particles()
    assert relerr(p["fHIp"], o.fHIp) <= 1e-4


def test_fortran_layout_roundtrip(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(12, 10, 8))
    ff = box.get_f_fortran()
    assert np.array_equal(np.transpose(ff, (0, 3, 2, 1)), o.f)
    box.set_f_fortran(ff * 0.5)
    assert np.array_equal(box.get_f(), o.f * 0.5)


@pytest.mark.parametrize("precision", [capi.LBM_PREC_F64, capi.LBM_PREC_F32])
def test_fortran_layout_page_locked(require_gpu, oracle_mod, precision):
    """Upload and download of the reference-layout populations from
    page-locked host memory (read and written by the GPU in place) give the
    same bits as the staged path from pageable memory."""
    import torch
    from multiphase_flow_codes_gb300._capi import dptr
    o, box = make_pair(oracle_mod, shape=(40, 20, 12), precision=precision)
    ff = box.get_f_fortran()                       # pageable: staged path
    n = ff.size
    pin = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    hp = np.ndarray(ff.shape, dtype=np.float64, buffer=pin, order="F")
    box._ck(box._L.lbm_download_f(box.handle, dptr(hp)), "download_f")
    assert np.array_equal(hp, ff)
    rng = np.random.default_rng(5)
    hp[...] = ff * (1.0 + 1e-3 * rng.standard_normal(ff.shape))
    box._ck(box._L.lbm_upload_f(box.handle, dptr(hp)), "upload_f")
    back = box.get_f_fortran()
    ref = hp.astype(np.float32).astype(np.float64) if precision == capi.LBM_PREC_F32 else hp
    assert np.array_equal(back, ref)
    box.close()


def test_page_locked_download_between_fused_steps(require_gpu, oracle_mod):
    """Between the FP64 plain path's fused steps the populations are stored
    in fixed point; a download to page-locked memory converts them on the way
    out (the same values as the staged download, which converts the buffer in
    place) and leaves the stored state alone, so steps with downloads in
    between follow the trajectory of steps without, bit for bit."""
    import torch
    from multiphase_flow_codes_gb300._capi import dptr
    _, a = make_pair(oracle_mod, shape=(40, 24, 16), npart=2, rad=4.0, rhopart=2.5)
    _, b = make_pair(oracle_mod, shape=(40, 24, 16), npart=2, rad=4.0, rhopart=2.5)
    a.set_variant(capi.LBM_VARIANT_DIRECT)
    b.set_variant(capi.LBM_VARIANT_DIRECT)
    n = 19 * 40 * 24 * 16
    pin = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()
    hp = np.ndarray((19, 40, 24, 16), dtype=np.float64, buffer=pin, order="F")
    for _ in range(4):
        a.step(1)
        b.step(1)
        a._ck(a._L.lbm_download_f(a.handle, dptr(hp)), "download_f")
    assert np.array_equal(a.get_f(), b.get_f())
    assert np.array_equal(hp, b.get_f_fortran())
    a.close()
    b.close()


def test_mass_momentum(require_gpu, oracle_mod):
    o, box = make_pair(oracle_mod, shape=(16, 16, 16))
    box.step(3)
    f = box.get_f()
    mm = box.mass_momentum()
    from conftest import CIX, CIY, CIZ
    ref = [f.sum(), np.tensordot(CIX, f, axes=(0, 0)).sum(), np.tensordot(CIY, f, axes=(0, 0)).sum(),
           np.tensordot(CIZ, f, axes=(0, 0)).sum()]
    assert np.allclose(mm, ref, atol=1e-12)


def _bounce_cases(o):
    """Counts of beads_collision's five interpolation cases over the oracle's
    links: (alpha <= 1/2: x - c solid, x - 2c solid, neither;
    alpha > 1/2: x - c solid, not)."""
    from conftest import CIX, CIY, CIZ
    part, node, ipop, alpha = oracle_links(o)
    nx, ny, nz = o.nx, o.ny, o.nz
    i, j, k = node % nx, (node // nx) % ny, node // (nx * ny)
    solid = o.ibnodes > 0

    def at(s):
        return solid[(k - s * CIZ[ipop]) % nz, (j - s * CIY[ipop]) % ny, (i - s * CIX[ipop]) % nx]

    s1, s2, low = at(1), at(2), alpha <= 0.5
    return [int((low & s1).sum()), int((low & ~s1 & s2).sum()), int((low & ~s1 & ~s2).sum()),
            int((~low & s1).sum()), int((~low & ~s1).sum())]


def test_bounce_cases_near_contact(require_gpu, oracle_mod):
    """Two spheres 0.6 lattice units apart (inside the lubrication range) and
    a third alone: the links in the gap see solid nodes at x - c and x - 2c,
    so every interpolation case of the bounce-back runs; populations, forces
    and torques against the oracle over 10 steps."""
    shape = (40, 36, 36)
    y = np.array([[12.2, 18.3, 17.9], [20.8, 18.6, 18.1], [30.0, 8.0, 26.0]])
    wp = np.array([[0.01, -0.01, 0.0], [-0.01, 0.01, 0.01], [0.0, 0.03, -0.02]])
    om = np.array([[0.0, 0.004, -0.002], [0.003, 0.0, 0.001], [0.0, 0.0, 0.005]])
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, *shape, 3, 4.0, 2.5)
    o = oracle_mod.OracleBox(cfg)
    u = inputs.spectral_velocity(shape[0], 4.0, 0.03, ny=shape[1], nz=shape[2])
    o.initpop(*u)
    o.macrovar()
    box = LBMBox(cfg)
    box.set_f(o.f.copy())
    box.macrovar()
    o.release_particles(y, wp, om)
    box.release_particles(y, wp, om)
    cases = _bounce_cases(o)
    assert min(cases) > 0, cases
    worst = {}
    for s in range(10):
        o.step(1)
        box.step(1)
        check_flags(o, box)
        for k, v in check_force_torque(o, box).items():
            worst[k] = max(worst.get(k, 0.0), v)
        p = box.get_particles()
        if s == 0:  # the pair starts inside the lubrication range (it is pushed apart)
            assert np.abs(o.flubp[:2]).max() > 0
        worst["flubp"] = max(worst.get("flubp", 0.0), relerr(p["flubp"], o.flubp[:3]))
        assert relerr(p["flubp"], o.flubp[:3]) <= TOL64
    print(f"\nnear contact, worst over 10 steps: {worst}")
    assert relerr(box.get_f(), o.f) <= TOL64
    p = box.get_particles()
    assert relerr(p["ypglb"], o.ypglb) <= TOL64
    assert relerr(p["omgp"], o.omgp) <= TOL64
    assert relerr(p["wp"], o.wp) <= TOL64
