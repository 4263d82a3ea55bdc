"""The C ABI library on the CPU host: it loads, exports every symbol the header
declares, has the reference's Params layout, and fails cleanly without a GPU.
No compute call is made here."""
import ctypes
import os
import re

import numpy as np
import pytest

from fluidgb import FlParams, FlStats, SIGNATURES, scenes

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "fluidgb.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_the_step_api():
    names = declared_functions()
    for required in ("fl_create", "fl_destroy", "fl_set_params", "fl_set_particles", "fl_get_particles",
                     "fl_step", "fl_step_device", "fl_apply_impulse", "fl_reset", "fl_get_grid", "fl_get_bins",
                     "fl_get_stats", "fl_save_state", "fl_load_state", "fl_last_error", "fl_solve_pressure"):
        assert required in names


def test_library_exports_every_declared_symbol(fluidlib):
    for name in declared_functions():
        assert hasattr(fluidlib, name), name
    assert set(declared_functions()) == set(SIGNATURES), "ctypes binding and header disagree"


def test_abi_version(fluidlib):
    assert fluidlib.fl_abi_version() == 1


# The reference's detailed GPU timing sections (gpu/timing.rs:32-59, FINE_SECTIONS)
# and CG categories (timing.rs:93, CG_CATS), in its order.
REFERENCE_SECTIONS = [
    "clear", "mark", "sort", "classify", "scatter", "normalize_u", "normalize_v", "normalize_w", "savevel_u",
    "savevel_v", "savevel_w", "forces_u", "forces_v", "forces_w", "bound_pre_u", "bound_pre_v", "bound_pre_w",
    "divergence", "cg_init", "gradient_u", "gradient_v", "gradient_w", "bound_post_u", "bound_post_v",
    "bound_post_w", "g2p", "cg_spmv", "cg_reduce", "cg_update", "cg_scalars",
]


def test_section_names_are_the_reference_sections(fluidlib):
    from fluidgb import _abi
    table = _abi.section_table(fluidlib)
    assert [n for n, _ in table] == REFERENCE_SECTIONS
    stage = dict(table)
    # the coarse rollup's boundaries (timing.rs PREP_END / FINISH_START): every
    # prep section is timed by a stage of the prep rollup, and so on
    prep_stages = {"sort", "classify", "scatter", "prep"}
    for n in REFERENCE_SECTIONS[:REFERENCE_SECTIONS.index("divergence")]:
        assert stage[n] in prep_stages, n
    for n in REFERENCE_SECTIONS[REFERENCE_SECTIONS.index("gradient_u"):REFERENCE_SECTIONS.index("g2p") + 1]:
        assert stage[n] in {"gradient", "g2p"}, n
    for n in ("cg_spmv", "cg_reduce", "cg_update", "cg_scalars"):
        assert stage[n] == "cg"
    assert fluidlib.fl_section_name(len(REFERENCE_SECTIONS)) is None
    assert fluidlib.fl_section_stage(len(REFERENCE_SECTIONS)) == -1


def test_params_layout_is_the_reference_uniform():
    # gpu/fluid.rs:25-39: 8 x vec4 = 128 bytes, then the extension block
    offs = {name: getattr(FlParams, name).offset for name, _ in FlParams._fields_}
    assert [offs[k] for k in ("dims", "geom", "phys", "origin", "grav", "spc", "cls", "gdim")] == \
        [0, 16, 32, 48, 64, 80, 96, 112]
    assert offs["pressure_tolerance"] == 128
    assert ctypes.sizeof(FlParams) == 160
    assert ctypes.sizeof(FlStats) == 40


def test_params_default_is_the_registry(fluidlib):
    p = FlParams()
    assert fluidlib.fl_params_default(ctypes.byref(p), 80, 40, 80, 2.0 / 64.0, None) == 0
    assert list(p.gdim[:3]) == [80, 40, 80]
    assert list(p.dims) == [80, 0, 30, 1]
    assert p.geom[2] == np.float32(1.0 / 120.0) and p.geom[3] == 65536.0
    assert p.phys[1] == 1000.0 and p.phys[2] == np.float32(0.9)
    assert p.origin[0] == np.float32(-80 * (2.0 / 64.0) / 2.0)
    assert p.cls[2] == 2.0 and p.spc[1] == np.float32(0.45)
    # the Python scene builder fills the same fields
    q = scenes.params_for(32, flip=0.9, iters=30, tol=0.0)
    r = FlParams()
    fluidlib.fl_params_default(ctypes.byref(r), 32, 32, 32, 1.0 / 32, (ctypes.c_float * 3)(0, 0, 0))
    for f in ("geom", "phys", "grav", "spc", "cls", "gdim"):
        assert list(getattr(q, f)) == list(getattr(r, f)), f


def test_invalid_arguments_are_rejected_without_a_device(fluidlib):
    h = ctypes.c_void_p()
    assert fluidlib.fl_create(None, 10, ctypes.byref(h)) == 1
    assert b"NULL" in fluidlib.fl_last_error(None)
    p = scenes.params_for(2)            # < 3 cells per axis
    assert fluidlib.fl_create(ctypes.byref(p), 10, ctypes.byref(h)) == 1
    p = scenes.params_for(16)
    p.reserved[0] = 7
    assert fluidlib.fl_create(ctypes.byref(p), 10, ctypes.byref(h)) == 1
    assert fluidlib.fl_step(None, 1) == 1
    assert fluidlib.fl_status_string(5) == b"FL_TIMEOUT"
    p = scenes.params_for(16)
    p.pressure_solver = 2               # neither FL_SOLVER_CG nor FL_SOLVER_MGPCG
    assert fluidlib.fl_create(ctypes.byref(p), 10, ctypes.byref(h)) == 1
    assert b"pressure_solver" in fluidlib.fl_last_error(None)
    # relaxation solver: arguments are checked before the device
    ct = np.zeros(16 ** 3, np.uint8)
    dv = np.zeros(16 ** 3, np.float32)
    out = np.zeros(16 ** 3, np.float32)
    ctp = ct.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    f32 = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert fluidlib.fl_relax_pressure(16, 16, 16, ctp, f32(dv), 1.0, 1.0, 1.0, 2, 10, f32(out)) == 1  # method
    assert fluidlib.fl_relax_pressure(16, 16, 16, None, f32(dv), 1.0, 1.0, 1.0, 0, 10, f32(out)) == 1
    assert fluidlib.fl_relax_pressure(2, 16, 16, ctp, f32(dv), 1.0, 1.0, 1.0, 0, 10, f32(out)) == 1
    assert fluidlib.fl_relax_pressure(16, 16, 16, ctp, f32(dv), 1.0, 0.0, 1.0, 0, 10, f32(out)) == 1  # rho
    # tape and replay entry points reject NULL handles
    assert fluidlib.fl_tape_set_adjoint_warm_start(None, 1) == 1
    assert fluidlib.fl_copy_pressure_device(None, None) == 1
    assert fluidlib.fl_step_replay(None, None, None) == 1


def test_create_without_gpu_reports_no_device(fluidlib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = scenes.params_for(16)
    h = ctypes.c_void_p()
    assert fluidlib.fl_create(ctypes.byref(p), 10, ctypes.byref(h)) == 6  # FL_NO_DEVICE
    assert not h.value


def test_header_compiles_as_c_and_links(fluidlib, tmp_path):
    """include/fluidgb.h is plain C (a cgo / bindgen consumer sees it that
    way): a C translation unit using the INTEGRATION example's calls compiles
    with -std=c99 -Wall -Werror and links against libfluidgb.so."""
    import shutil
    import subprocess
    from fluidgb import _abi
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use.c"
    src.write_text(r'''
#include <stdio.h>
#include "fluidgb.h"
int main(void) {
    fl_params p;
    float origin[3] = {0.0f, 0.0f, 0.0f};
    fl_handle* h = 0;
    if (fl_params_default(&p, 32, 32, 32, 1.0f / 32, origin) != FL_OK) return 1;
    p.pressure_solver = FL_SOLVER_CG;
    p.cg_precision = FL_CG_F64;
    if (fl_create(&p, 16, &h) == FL_OK) {
        fl_step(h, 1);
        fl_destroy(h);
    } else {
        printf("%s\n", fl_last_error(0));
    }
    printf("abi %u\n", fl_abi_version());
    return 0;
}
''')
    exe = tmp_path / "use"
    lib_dir = os.path.dirname(_abi.LIB_PATH)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.dirname(HEADER), str(src),
                        "-L", lib_dir, "-l:" + os.path.basename(_abi.LIB_PATH), "-Wl,-rpath," + lib_dir,
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and "abi 1" in out.stdout, out.stdout + out.stderr
