"""The C ABI library loads without a GPU, exports every symbol include/lbm.h
declares, and its configuration helpers reproduce the reference's values."""

import ctypes as C
import math
import re
from pathlib import Path

import pytest

from multiphase_flow_codes_gb300 import _capi as capi

HEADER = Path(__file__).resolve().parents[1] / "include" / "lbm.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(engine_lib):
    names = declared_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(engine_lib, n)]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert set(names) <= set(capi.SIGNATURES), set(names) - set(capi.SIGNATURES)


def test_config_struct_layout(engine_lib):
    assert C.sizeof(capi.lbm_config) == 16 * 4 + 20 * 8
    assert engine_lib.lbm_version() == 1


def test_box_preset_matches_reference(engine_lib):
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 64, 64, 64, 16, 4.5, 5.0)
    volp = 4.0 / 3.0 * math.pi * 4.5 ** 3
    assert cfg.mrt_type == 1 and cfg.forcing == capi.LBM_FORCING_STOCHASTIC
    assert cfg.iseedf == 232300 and cfg.iseedp == 12345
    assert cfg.fpc == pytest.approx(volp * 9.8 / 2500.0, rel=1e-15)
    assert cfg.stf0 == 0.025 and cfg.stf1 == 0.002
    assert cfg.vscale == 2.037183272e-3


def test_channel_preset_matches_reference(engine_lib):
    nx = 249
    cfg = capi.config_init(capi.LBM_PRESET_CHANNEL, nx, 400, 200, 10, 5.0, 1.0)
    ustar = 2.0 * 180.0 * 0.0036 / nx
    force_in_y = 2.0 * ustar * ustar / nx
    ystar = 0.0036 / ustar
    volp = 4.0 / 3.0 * math.pi * 125.0
    assert cfg.mrt_type == 2 and cfg.boundary == capi.LBM_BC_XWALLS
    assert cfg.force_y == pytest.approx(force_in_y, rel=1e-14)
    assert cfg.fpc == pytest.approx(volp * ustar * ustar / ystar, rel=1e-14)
    assert cfg.body_force_y == pytest.approx(volp * force_in_y, rel=1e-14)


def test_footprint_and_bad_arguments(engine_lib):
    cfg = capi.config_init(capi.LBM_PRESET_BOX, 256, 256, 256, 1000, 4.0, 2.5)
    b = capi.footprint(cfg)
    assert 5.0e9 < b < 8.0e9
    bad = capi.lbm_config()
    h = C.c_void_p()
    assert engine_lib.lbm_create(C.byref(bad), C.byref(h)) == capi.LBM_ERR_ARG
    with pytest.raises(capi.LBMError):
        capi.config_init(capi.LBM_PRESET_BOX, 2, 2, 2, 0, 1.0, 1.0)


@pytest.mark.gpu
def test_fma_throughput_probe(engine_lib, require_gpu):
    """The FP64 and FP32 FMA rates the roofline of the fused kernel is quoted against."""
    f64, f32 = C.c_double(0.0), C.c_double(0.0)
    assert engine_lib.lbm_fma_throughput(capi.LBM_PREC_F64, C.byref(f64)) == capi.LBM_OK
    assert engine_lib.lbm_fma_throughput(capi.LBM_PREC_F32, C.byref(f32)) == capi.LBM_OK
    assert 0.1 < f64.value < 200.0
    assert f32.value > f64.value
    assert engine_lib.lbm_fma_throughput(capi.LBM_PREC_F64, None) == capi.LBM_ERR_ARG


@pytest.mark.parametrize("preset,dims,npart,rad,ratio", [
    (capi.LBM_PRESET_BOX, (64, 64, 64), 16, 4.5, 5.0),
    (capi.LBM_PRESET_BOX, (256, 256, 256), 1000, 4.0, 2.5),
    (capi.LBM_PRESET_CHANNEL, (96, 64, 128), 40, 4.0, 1.0),
])
def test_oracle_config_equals_engine_config(engine_lib, preset, dims, npart, rad, ratio):
    """The CPU reference leg of the benchmark builds its parameter block
    without the engine library; every field must equal the engine's."""
    from oracle import config as ocfg
    a = capi.config_init(preset, *dims, npart, rad, ratio)
    b = ocfg.config_init(preset, *dims, npart, rad, ratio)
    assert C.sizeof(ocfg.lbm_config) == C.sizeof(capi.lbm_config)
    assert bytes(a) == bytes(b)
