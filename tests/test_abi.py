"""The C-ABI library builds for sm_103a, loads, and exports every symbol the header declares.

No CUDA work is launched here (no GPU in the CPU suite).
"""

import ctypes
import os
import re
import subprocess

import pytest

from torchfsm_gb300 import _lib, build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "torchfsm_gb300.h")


@pytest.fixture(scope="module")
def libpath():
    return build.build()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(fsm_\w+)\s*\(", text)))


def test_header_declares_the_binding_exports():
    assert declared_functions() == sorted(_lib.EXPORTS)


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT\s+(fsm_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_library_loads_and_reports_version(libpath):
    lib = _lib.load(libpath)
    assert lib.fsm_abi_version() == 1
    buf = ctypes.create_string_buffer(64)
    assert lib.fsm_last_error(buf, 64) == 0


def test_invalid_arguments_return_status_without_gpu(libpath):
    lib = _lib.load(libpath)
    out = ctypes.c_void_p()
    # null descriptors are rejected before any CUDA call
    assert lib.fsm_plan_create(None, None, 0.1, None, ctypes.byref(out)) == _lib.FSM_ERR_INVALID
    assert "null" in _lib.last_error()
    mesh = _lib.FsmMeshDesc()
    mesh.ndim = 1
    mesh.n[0] = 100  # not a power of two
    mesh.length[0] = 1.0
    prog = _lib.FsmProgramDesc()
    prog.n_channel = 1
    prog.integrator = _lib.FSM_SETDRK4
    prog.nonlinear = _lib.FSM_NL_CONVECTION
    assert lib.fsm_plan_create(ctypes.byref(mesh), ctypes.byref(prog), 0.1, None, ctypes.byref(out)) == \
        _lib.FSM_ERR_UNSUPPORTED
    mesh.n[0] = 128
    prog.nonlinear = _lib.FSM_NL_VORTICITY  # needs 2D
    assert lib.fsm_plan_create(ctypes.byref(mesh), ctypes.byref(prog), 0.1, None, ctypes.byref(out)) == \
        _lib.FSM_ERR_INVALID


def test_serving_engine_rejects_null_arguments_without_gpu(libpath):
    lib = _lib.load(libpath)
    out = ctypes.c_void_p()
    assert lib.fsm_serve_create(None, 4, 8, None, None, 0, 0, 0.0, None, ctypes.byref(out)) == _lib.FSM_ERR_INVALID
    assert "serve_create" in _lib.last_error()
    nb = ctypes.c_size_t()
    assert lib.fsm_serve_workspace_bytes(None, 4, 8, ctypes.byref(nb)) == _lib.FSM_ERR_INVALID
    grp = ctypes.c_void_p()
    assert lib.fsm_serve_group_create(None, 2, 0.0, ctypes.byref(grp)) == _lib.FSM_ERR_INVALID
    assert lib.fsm_serve_group_tick(None, ctypes.byref(k := ctypes.c_int32())) == _lib.FSM_ERR_INVALID
    assert lib.fsm_serve_group_destroy(None) == _lib.FSM_OK
    assert lib.fsm_serve_submit(None, 1, 1, 1, 0.1, None, None) == _lib.FSM_ERR_INVALID
    k = ctypes.c_int32()
    assert lib.fsm_serve_tick(None, ctypes.byref(k)) == _lib.FSM_ERR_INVALID
    n, busy = ctypes.c_int32(), ctypes.c_int32()
    assert lib.fsm_serve_poll(None, 0, None, 0, ctypes.byref(n), ctypes.byref(busy)) == _lib.FSM_ERR_INVALID
    assert lib.fsm_serve_cancel(None, 1) == _lib.FSM_ERR_INVALID
    st = ctypes.c_int32()
    assert lib.fsm_serve_request_status(None, 1, ctypes.byref(st), None) == _lib.FSM_ERR_INVALID
    stats = (ctypes.c_int64 * _lib.FSM_SERVE_NSTATS)()
    assert lib.fsm_serve_stats(None, stats, _lib.FSM_SERVE_NSTATS) == _lib.FSM_ERR_INVALID
    assert lib.fsm_serve_destroy(None) == _lib.FSM_OK


def test_step_adjoint_rejects_null_arguments_without_gpu(libpath):
    lib = _lib.load(libpath)
    n = ctypes.c_size_t()
    assert lib.fsm_step_adjoint_workspace_bytes(None, 1, ctypes.byref(n)) == _lib.FSM_ERR_INVALID
    assert lib.fsm_step_adjoint(None, 1, None, None, None, None, None, 0, None) == _lib.FSM_ERR_INVALID
    assert "step_adjoint" in _lib.last_error()


def test_descriptor_layouts_match_the_header(tmp_path):
    """The ctypes descriptors the binding passes have the header's field offsets and sizes
    (a C program compiled with the host compiler reports offsetof / sizeof)."""
    import shutil

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"FsmMeshDesc": _lib.FsmMeshDesc, "FsmProgramDesc": _lib.FsmProgramDesc}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "torchfsm_gb300.h"', "int main(void) {"]
    for name, cls in structs.items():
        lines.append(f'  printf("{name} sizeof %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name} {field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in filter(None, out):
        struct, field, value = line.split()
        got[(struct, field)] = int(value)
    for name, cls in structs.items():
        assert got[(name, "sizeof")] == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert got[(name, field)] == getattr(cls, field).offset, (name, field)


def test_binding_argument_counts_match_the_header(libpath):
    """Every entry point the binding declares argtypes for takes as many arguments as its
    prototype in the header."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    protos = dict(re.findall(r"\bint\s+(fsm_\w+)\s*\(([^)]*)\)", text))
    lib = _lib.load(libpath)
    checked = 0
    for name, params in protos.items():
        argtypes = getattr(lib, name).argtypes
        if argtypes is None:
            continue
        params = params.strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        assert len(argtypes) == n, (name, len(argtypes), n)
        checked += 1
    assert checked >= len(protos) - 2  # the version and error queries may keep ctypes defaults
