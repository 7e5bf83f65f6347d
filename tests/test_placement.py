"""lbm_place_particles: initpartpos on the host, bit for bit.

The engine's placement (the one lbm_init_particles and the serving loop use)
tests, per round, only the pairs that can have changed, found through a cell
grid; the reference's ovlpchk tests every pair.  These CPU tests hold it to
the all-pairs restatements: the Python ``inputs.initpartpos`` on small cases
and the oracle's ``initpartpos`` (3DBox.../partlib.f90:1-80,
3DChannel.../partlib.f90:10-24) on dense ones that take thousands of rounds,
including grids with fewer than three cells on an axis and the channel's
walls.  No GPU is needed.
"""

import numpy as np
import pytest

from multiphase_flow_codes_gb300 import _capi as capi
from multiphase_flow_codes_gb300 import inputs


def cfg_for(shape, npart, rad, channel, seed):
    preset = capi.LBM_PRESET_CHANNEL if channel else capi.LBM_PRESET_BOX
    cfg = capi.config_init(preset, *shape, npart, rad, 1.0)
    cfg.iseedp = seed
    return cfg


@pytest.mark.parametrize("shape,npart,rad,channel,seed", [
    ((48, 48, 48), 20, 4.0, False, 12345),
    ((48, 48, 48), 20, 4.0, True, 12345),
    ((40, 24, 56), 30, 3.0, False, 777),
    ((32, 40, 24), 25, 2.5, True, 4242),
    ((16, 64, 64), 12, 2.5, False, 99),   # one cell along x (16 < 3 cut-offs)
    ((64, 20, 64), 15, 3.0, True, 5),     # one cell along y
])
def test_placement_matches_python(engine_lib, shape, npart, rad, channel, seed):
    cfg = cfg_for(shape, npart, rad, channel, seed)
    got = capi.place_particles(cfg, npart, seed)
    ref = inputs.initpartpos(*shape, npart, rad, cfg.mingap, seed=seed, channel=channel,
                             mingap_w=cfg.mingap_w)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape,npart,rad,channel,seed", [
    ((64, 64, 112), 222, 4.0, True, 10_001),   # ~2000 rounds
    ((64, 64, 64), 150, 4.0, False, 31),
    ((96, 72, 80), 300, 4.0, True, 8),
    ((24, 96, 96), 140, 3.0, False, 17),
])
def test_dense_placement_matches_oracle(engine_lib, oracle_mod, shape, npart, rad, channel, seed):
    cfg = cfg_for(shape, npart, rad, channel, seed)
    got = capi.place_particles(cfg, npart, seed)
    o = oracle_mod.OracleBox(cfg)
    assert o.initpartpos(npart) == 0
    assert np.array_equal(got, o.ypglb[:npart])
    o.close()


def test_placement_gives_up_like_the_reference(engine_lib):
    shape, npart, rad = (32, 32, 32), 40, 4.0   # far too dense to place
    cfg = cfg_for(shape, npart, rad, False, 3)
    with pytest.raises(capi.LBMError) as e:
        capi.place_particles(cfg, npart, 3, max_rounds=50)
    assert e.value.code == capi.LBM_ERR_OVERLAP
    with pytest.raises(RuntimeError):
        inputs.initpartpos(*shape, npart, rad, cfg.mingap, seed=3, max_rounds=50)
