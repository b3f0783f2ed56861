"""The C++ drop-in header (include/rd_lagrange_euler_view.hpp): the
reference's initialiser restated in it (CPU) and a main.cpp-style driver
linked against the CUDA library (GPU)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, b_scale, golden, rel, rel_floor

INC = os.path.join(REPO, "include")
CPP = os.path.join(REPO, "tests", "cpp")


def test_reference_initialiser_is_bit_exact(tmp_path):
    exe = tmp_path / "init_positions"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", INC, os.path.join(CPP, "init_positions.cpp"), "-o",
                           str(exe)])
    out = tmp_path / "x.bin"
    more = subprocess.check_output([str(exe), str(out)], text=True)
    assert int(more) == 3  # the reference prints "3 more!!!" for its own scene
    rec = np.fromfile(out, np.float32).reshape(-1, 4)
    g = golden("ref_scene_20.npz")
    assert np.array_equal(rec[:, :3], g["x0"])
    assert np.array_equal(rec[:, 3], g["m0"])


def test_exchange_arrays_round_trip_bit_exact_on_host_threads(tmp_path):
    """Particle <-> exchange arrays of the drop-in, split over host threads for
    large counts, against a plain one-thread conversion (no GPU needed)."""
    exe = tmp_path / "facade_exchange"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-pthread", "-I", INC,
                           os.path.join(CPP, "facade_exchange.cpp"), "-o", str(exe)])
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["stages", "fused"])
def test_cpp_driver_matches_reference_scene(built_pkg, tmp_path, mode):
    exe = tmp_path / "drive"
    libdir = os.path.dirname(built_pkg.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-pthread", "-I", INC, os.path.join(CPP, "main_reference_scene.cpp"),
                           "-L", libdir, "-l:librd_mpm.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)])
    out = tmp_path / "state.bin"
    subprocess.check_call([str(exe), str(out), mode])
    rec = np.fromfile(out, np.float32).reshape(-1, 34)
    g = golden("ref_scene_20.npz")
    assert rel(rec[:, 0:3], g["s1_x"]) < 1e-5
    assert rel(rec[:, 3:6], g["s1_v"]) < 1e-5
    assert rel_floor(rec[:, 6:15], g["s1_B"], b_scale(g["s1_v"], 0.05)) < 1e-5
    assert rel(rec[:, 15:24], g["s1_FE"]) < 1e-5
    assert rel(rec[:, 24:33], g["s1_FP"]) < 1e-5
    assert rel(rec[:, 33], g["vol0"]) < 1e-6


def test_cpp_driver_compiles_with_the_reference_logging_calls(tmp_path):
    """main.cpp:51 (MPM.setLevel(MaterialPointMethod::DEFAULT_LOG_LEVEL_MPM))
    and the rest of main.cpp:48-54 compile against the drop-in header."""
    obj = tmp_path / "drive.o"
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-c", "-I", INC, os.path.join(CPP, "main_reference_scene.cpp"),
                           "-o", str(obj)])


@pytest.mark.gpu
def test_cpp_driver_logs_like_the_reference(built_pkg, tmp_path):
    """At INFO the stage calls print the reference's diagnostics (its
    material_point_method.cpp:61-62,122-125,140-141,329); at the default
    WARNING level nothing is printed for this scene."""
    exe = tmp_path / "drive"
    libdir = os.path.dirname(built_pkg.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-pthread", "-I", INC, os.path.join(CPP, "main_reference_scene.cpp"),
                           "-L", libdir, "-l:librd_mpm.so", f"-Wl,-rpath,{libdir}", "-o", str(exe)])
    quiet = subprocess.run([str(exe), str(tmp_path / "a.bin"), "stages"], capture_output=True, text=True, check=True)
    assert quiet.stdout == ""
    loud = subprocess.run([str(exe), str(tmp_path / "b.bin"), "stages", "info"], capture_output=True, text=True,
                          check=True)
    lines = loud.stdout.splitlines()
    heads = [ln.split(" is: ")[0] for ln in lines if " is: " in ln]
    assert heads[:2] == ["Particles momentum", "Average PPC"]
    assert heads.count("ParticlesMomentum") == 2 and heads.count("GridMomentum") == 2
    assert "Average cell density" in heads and "Average particle density" in heads
    assert "Average deformation gradient" in heads
    # 2147 particles of mass 6e-5 moving at (0, -200, 0): momentum (0, -25.764, 0)
    pm = [ln for ln in lines if ln.startswith("Particles momentum is: ")][0].split(": ")[1].split()
    assert abs(float(pm[1]) + 2147 * 6e-5 * 200) < 1e-3 and abs(float(pm[0])) < 1e-6
    ppc = float([ln for ln in lines if ln.startswith("Average PPC is: ")][0].split(": ")[1])
    assert 4.0 < ppc < 8.0
    assert "GridMomentum != ParticlesMomentum" not in loud.stdout
