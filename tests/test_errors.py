"""Status codes where the reference stops (partlib.f90:2634-2646 and others).

Every failure here is made on the host side of the GPU: overlapping or
non-finite particle positions, a link capacity too small, a box above the
32-bit node limit.  The kernels detect them with bounds-checked code and
report them through the context's status word; the context stays usable.
"""

import ctypes as C

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import LBMError

pytestmark = pytest.mark.gpu


def _box(n=32, npart=2, rad=4.0, link_capacity=0):
    from multiphase_flow_codes_gb300.engine import LBMBox
    cfg = capi.config_init(capi.LBM_PRESET_BOX, n, n, n, npart, rad, 2.5)
    if link_capacity:
        cfg.link_capacity = link_capacity
    box = LBMBox(cfg)
    z = np.zeros((n, n, n))
    box.initpop(z, z, z)
    box.macrovar()
    return box


def test_overlap_after_move_is_reported(require_gpu, oracle_mod):
    """Two spheres closer than 2R: the reference stops after beads_move's
    redistribute (ovlpchk); here the step reports LBM_ERR_OVERLAP."""
    box = _box()
    y = np.array([[10.0, 16.0, 16.0], [15.0, 16.0, 16.0]])  # 5 apart, R = 4
    box.release_particles(y)
    with pytest.raises(LBMError) as e:
        box.step(1)
        box.synchronize()
    assert e.value.code == capi.LBM_ERR_OVERLAP
    # the oracle agrees on the same input
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 32, 32, 32, 2, 4.0, 2.5)
    o = oracle_mod.OracleBox(cfg)
    z = np.zeros((32, 32, 32))
    o.initpop(z, z, z)
    o.macrovar()
    o.release_particles(y)
    assert o.step(1) == capi.LBM_ERR_OVERLAP


def test_link_capacity_is_reported(require_gpu):
    box = _box(link_capacity=16)
    with pytest.raises(LBMError) as e:
        box.release_particles(np.array([[8.0, 8.0, 8.0], [24.0, 24.0, 24.0]]))
        box.step(1)
        box.synchronize()
    assert e.value.code == capi.LBM_ERR_CAPACITY


def test_nonfinite_particle_is_reported(require_gpu):
    box = _box()
    with pytest.raises(LBMError) as e:
        box.release_particles(np.array([[8.0, np.nan, 8.0], [24.0, 24.0, 24.0]]))
        box.step(1)
        box.synchronize()
    assert e.value.code == capi.LBM_ERR_NONFINITE


def test_context_usable_after_error(require_gpu):
    """After a reported error the caller can put a valid state back and go on."""
    box = _box()
    with pytest.raises(LBMError):
        box.release_particles(np.array([[10.0, 16.0, 16.0], [15.0, 16.0, 16.0]]))
        box.step(1)
        box.synchronize()
    box.release_particles(np.array([[8.0, 8.0, 8.0], [24.0, 24.0, 24.0]]))
    box.step(3)
    box.synchronize()
    assert np.isfinite(box.get_f()).all()


def test_box_above_node_limit_rejected(require_gpu):
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 512, 512, 256, 0, 4.0, 1.0)  # 2^26 nodes
    h = C.c_void_p()
    assert capi.lib().lbm_create(C.byref(cfg), C.byref(h)) == capi.LBM_ERR_ARG


def test_small_box_and_no_particles(require_gpu, oracle_mod):
    """The smallest box the forcing accepts (6 in y and z), no particles."""
    from conftest import relerr
    from test_gpu_parity import TOL64, make_pair
    o, box = make_pair(oracle_mod, shape=(8, 6, 6), npart=0, urms=0.02, k0=2.0)
    for _ in range(5):
        o.step(1)
        box.step(1)
    assert relerr(box.get_f(), o.f) <= TOL64
