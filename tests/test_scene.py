"""Scene presets, particle budgets and the seeded lattice against the
reference's own scene tests (app/crates/fluid-lab/src/scene/mod.rs:463-700)
and the oracle's sequential restatement of generate_particles
(gpu/fluid.rs:1838-1913).  Host functions of the C ABI: no device needed."""
import ctypes

import numpy as np
import pytest

from fluidgb import FlParams
from fluidgb._abi import (FL_PRESET_DAM_BREAK, FL_PRESET_DOUBLE_SPLASH, FL_PRESET_FALLING_BLOB, scene_blocks,
                          scene_particle_count, seed_count, seeded_fraction)

PRESETS = (FL_PRESET_FALLING_BLOB, FL_PRESET_DAM_BREAK, FL_PRESET_DOUBLE_SPLASH)
DEFAULT_DROP = 0.72   # scene/mod.rs:10, used by the reference's preset_blocks tests
REGISTRY_DROP = 1.0   # the registry default of scene.drop_height (settings/mod.rs:428-437)
H = 2.0 / 64.0  # sim/mod.rs:26


@pytest.fixture
def lib(fluidlib):
    return fluidlib


def test_preset_seeded_fraction_keeps_authored_scale(lib):
    # scene/mod.rs:603-619
    for preset, fill, expected in ((FL_PRESET_FALLING_BLOB, 0.2, 0.199888), (FL_PRESET_FALLING_BLOB, 0.5, 0.499720),
                                   (FL_PRESET_DAM_BREAK, 0.5, 0.163170), (FL_PRESET_DOUBLE_SPLASH, 0.5, 0.173280)):
        frac = seeded_fraction(scene_blocks(preset, DEFAULT_DROP, fill, lib), lib)
        assert abs(frac - expected) < 0.005, (preset, fill, frac)
        assert abs(frac - expected) < 1e-5, (preset, fill, frac)  # the reference's printed values


def test_default_density_derives_count_from_seeded_cells(lib):
    # scene/mod.rs:513-523: registry defaults (80x40x80, density 10, falling blob, 20% fill)
    blocks = scene_blocks(FL_PRESET_FALLING_BLOB, REGISTRY_DROP, 0.2, lib)
    assert 511_000 <= scene_particle_count((80, 40, 80), blocks, 10.0, 0, lib) <= 513_000


def test_density_scales_count_with_grid_resolution(lib):
    # scene/mod.rs:525-535
    blocks = scene_blocks(FL_PRESET_FALLING_BLOB, REGISTRY_DROP, 0.2, lib)
    assert 1_305_000 <= scene_particle_count((128, 40, 128), blocks, 10.0, 0, lib) <= 1_315_000


def test_nonzero_particle_count_override_wins_over_density(lib):
    blocks = scene_blocks(FL_PRESET_FALLING_BLOB, REGISTRY_DROP, 0.2, lib)
    assert scene_particle_count((80, 40, 80), blocks, 10.0, 500_000, lib) == 500_000


def test_falling_blob_uses_drop_height(lib):
    low = scene_blocks(FL_PRESET_FALLING_BLOB, 0.0, 0.2, lib)[0]
    high = scene_blocks(FL_PRESET_FALLING_BLOB, 1.0, 0.2, lib)[0]
    assert abs(low.min[1]) < 1e-6
    assert high.min[1] > low.min[1] + 0.25
    assert abs(high.max[1] - 1.0) < 1e-6


def test_default_fill_level_is_falling_blob(lib):
    b = scene_blocks(FL_PRESET_FALLING_BLOB, DEFAULT_DROP, 0.2, lib)[0]  # scene_for(.., DEFAULT_DROP_HEIGHT)
    assert b.min[1] > 0.0 and b.max[1] < 1.0
    assert abs(seeded_fraction([b], lib) - 0.2) < 0.01


def test_double_splash_drop_height_clamps_inside_tank(lib):
    for dh in (0.0, 1.0):
        for b in scene_blocks(FL_PRESET_DOUBLE_SPLASH, dh, 0.2, lib):
            assert b.min[1] >= -1e-6 and b.max[1] <= 1.0 + 1e-6 and b.max[1] > b.min[1]


def test_dam_break_ignores_drop_height(lib):
    low = scene_blocks(FL_PRESET_DAM_BREAK, 0.0, 0.2, lib)[0]
    high = scene_blocks(FL_PRESET_DAM_BREAK, 1.0, 0.2, lib)[0]
    assert abs(low.min[1]) < 1e-6
    assert abs(high.min[1] - low.min[1]) < 1e-6 and abs(high.max[1] - low.max[1]) < 1e-6


def test_full_fill_uses_preset_authored_max_not_whole_tank(lib):
    # scene/mod.rs:560-569: registry defaults with scene.fill_level = 100
    frac = seeded_fraction(scene_blocks(FL_PRESET_FALLING_BLOB, REGISTRY_DROP, 1.0, lib), lib)
    assert 0.55 <= frac <= 0.75


def test_zero_fill_keeps_minimum_viable_seed(lib):
    for preset in PRESETS:
        blocks = scene_blocks(preset, DEFAULT_DROP, 0.0, lib)
        assert blocks and seeded_fraction(blocks, lib) > 0.0
        reg = scene_blocks(preset, REGISTRY_DROP, 0.0, lib)
        assert scene_particle_count((80, 40, 80), reg, 8.0, 0, lib) == 1024


def test_fill_level_is_monotone_in_seeded_fraction_and_count(lib):
    for preset in PRESETS:
        last_frac, last_count = -1.0, 0
        for fill in (0.1, 0.2, 0.5, 1.0):
            blocks = scene_blocks(preset, DEFAULT_DROP, fill, lib)
            frac = seeded_fraction(blocks, lib)
            count = scene_particle_count((64, 64, 64), blocks, 8.0, 0, lib)
            assert frac > last_frac + 1e-6 and count >= last_count
            last_frac, last_count = frac, count


def test_default_scene_fill_is_roughly_linear_before_clamping(lib):
    f20 = seeded_fraction(scene_blocks(FL_PRESET_FALLING_BLOB, DEFAULT_DROP, 0.2, lib), lib)
    f50 = seeded_fraction(scene_blocks(FL_PRESET_FALLING_BLOB, DEFAULT_DROP, 0.5, lib), lib)
    assert abs(f20 - 0.2) < 0.001 and 2.4 <= f50 / f20 <= 2.6


def default_params(lib, n3):
    p = FlParams()
    assert lib.fl_params_default(ctypes.byref(p), n3[0], n3[1], n3[2], H, None) == 0
    return p


@pytest.mark.parametrize("preset", PRESETS)
def test_seed_count_matches_the_sequential_layout(lib, oracle, preset):
    p = default_params(lib, (80, 40, 80))
    blocks = scene_blocks(preset, REGISTRY_DROP, 0.2, lib)
    budget = scene_particle_count((80, 40, 80), blocks, 10.0, 0, lib)
    n_ref, _ = oracle.ref_generate_particles(p, blocks, budget, 0)
    assert seed_count(p, blocks, budget, lib) == n_ref
    assert abs(n_ref - budget) < 0.1 * budget
