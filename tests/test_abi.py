"""CPU tests of the C ABI boundary: the header, the library's exported symbols,
struct layouts as ctypes sees them, and argument validation that needs no GPU."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import REPO, gpu_available

HEADER = os.path.join(REPO, "include", "rd_mpm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(rd_[a-z_0-9]+)\s*\(", text))


def test_header_declares_exactly_the_exports(pkg):
    assert declared_functions() == set(pkg.EXPORTS)


def test_missing_library_fails_loudly(pkg, monkeypatch):
    """No CPU fallback: without the built CUDA library every call raises."""
    monkeypatch.setattr(pkg, "_LIB", None)
    monkeypatch.setattr(pkg, "LIB_PATH", os.path.join(REPO, "no_such_dir", "librd_mpm.so"))
    with pytest.raises(RuntimeError, match="not built"):
        pkg.lib()
    with pytest.raises(RuntimeError, match="not built"):
        pkg.Simulation(pkg.make_params(16, 16, 16, 8, 1.0 / 16))


def test_library_loads_and_exports_every_declared_symbol(built_pkg):
    L = built_pkg.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", built_pkg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (rd_[a-z_0-9]+)\b", out))
    assert declared_functions() <= exported


def _c_layout(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(r"""
#include <stdio.h>
#include <stddef.h>
#include "rd_mpm.h"
#define F(s, m) printf(#s "." #m " %zu\n", offsetof(s, m));
int main(void) {
    printf("rd_params %zu\n", sizeof(rd_params));
    printf("rd_particles %zu\n", sizeof(rd_particles));
    F(rd_params, max_i) F(rd_params, max_j) F(rd_params, max_k) F(rd_params, num_particles) F(rd_params, h) F(rd_params, E) F(rd_params, nu)
    F(rd_params, xi) F(rd_params, theta_c) F(rd_params, theta_s) F(rd_params, gravity) F(rd_params, bc)
    F(rd_params, bc_width) F(rd_params, lagged_b) F(rd_params, track_fp) F(rd_params, precision)
    F(rd_params, device)
    F(rd_particles, x) F(rd_particles, v) F(rd_particles, B) F(rd_particles, FE) F(rd_particles, FP)
    F(rd_particles, Jp) F(rd_particles, mass) F(rd_particles, volume)
    return 0;
}
""")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True)
    return dict((k, int(v)) for k, v in (line.split() for line in out.strip().splitlines()))


def test_c_example_compiles_and_links_as_c99(built_pkg, tmp_path):
    """The integration guide's C example (tests/cpp/abi_example.c) builds
    against the header alone, as C99 with warnings as errors, and links
    against the library."""
    exe = tmp_path / "abi_example"
    libdir = os.path.dirname(built_pkg.LIB_PATH)
    subprocess.check_call(["gcc", "-std=c99", "-O2", "-Wall", "-Wextra", "-Werror", "-I",
                           os.path.join(REPO, "include"), os.path.join(REPO, "tests", "cpp", "abi_example.c"),
                           "-L", libdir, "-l:librd_mpm.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)])
    assert exe.exists()


def test_ctypes_structs_match_c_layout(pkg, tmp_path):
    c = _c_layout(tmp_path)
    assert c["rd_params"] == ctypes.sizeof(pkg.Params)
    assert c["rd_particles"] == ctypes.sizeof(pkg._Particles)
    for name, _ in pkg.Params._fields_:
        assert c[f"rd_params.{name}"] == getattr(pkg.Params, name).offset, name
    for name, _ in pkg._Particles._fields_:
        assert c[f"rd_particles.{name}"] == getattr(pkg._Particles, name).offset, name


def test_default_params_are_the_reference_constants(built_pkg):
    p = built_pkg.default_params()
    assert (p.max_i, p.max_j, p.max_k, p.num_particles) == (20, 20, 20, 2147)  # main.cpp:203-205
    assert p.h == pytest.approx(0.05)
    assert p.E == pytest.approx(1.4e5) and p.nu == pytest.approx(0.2) and p.xi == 10.0
    assert p.theta_c == pytest.approx(2.5e-2) and p.theta_s == pytest.approx(5e-3)
    assert tuple(p.gravity) == (0.0, -9.8, 0.0)
    assert p.lagged_b == 1 and p.bc == built_pkg.RD_BC_NONE


def test_create_rejects_bad_arguments_before_touching_the_device(built_pkg):
    L = built_pkg.lib()
    h = ctypes.c_void_p()
    assert L.rd_create(None, ctypes.byref(h)) == built_pkg.RD_INVALID_ARG
    for bad in (dict(max_i=4), dict(num_particles=-1), dict(h=0.0), dict(precision=7), dict(bc_width=-1)):
        p = built_pkg.make_params(16, 16, 16, 10, 1 / 16)
        for k, v in bad.items():
            setattr(p, k, v)
        assert L.rd_create(ctypes.byref(p), ctypes.byref(h)) == built_pkg.RD_INVALID_ARG, bad
    for fn in ("rd_destroy", "rd_init_volumes", "rd_synchronize", "rd_clear_flags"):
        assert getattr(L, fn)(None) == built_pkg.RD_INVALID_ARG, fn


def test_create_without_a_device_fails_cleanly(built_pkg):
    if gpu_available():
        pytest.skip("a GPU is present")
    L = built_pkg.lib()
    h = ctypes.c_void_p()
    p = built_pkg.make_params(16, 16, 16, 10, 1 / 16)
    assert L.rd_create(ctypes.byref(p), ctypes.byref(h)) == built_pkg.RD_CUDA_ERROR
    assert not h.value
