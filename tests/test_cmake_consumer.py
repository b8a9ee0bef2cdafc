"""A CMake host model linking the GPU mechanism libraries, on any host.

mkpp_gb300/cmake/MKPPGpuMechanism.cmake is the counterpart of the
reference's mkpp_add_compiled_mechanism
(src/mkpp_host/cmake/MKPPCompiledMechanism.cmake:9-53).  A small CMake
project includes it and builds two programs.  The C ABI contract program
(tests/capi/c_abi_contract.c) links a mechanism target made by
mkpp_gpu_add_mechanism.  The registry checker (tests/registry/
registry_check.cpp) links mkpp_gb300::registry, with no MKPP_GB300_LIB_DIR in
its environment, so it finds the libraries through the directory the
module compiles in.  Neither program makes a CUDA call.  A mechanism without
a plan stops at configure time with the reference's "FATAL ERROR" prefix.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
MODULE = ROOT / "mkpp_gb300" / "cmake" / "MKPPGpuMechanism.cmake"

PROJECT = """\
cmake_minimum_required(VERSION 3.20)
project(mkpp_consumer C CXX)
include("{module}")
mkpp_gpu_add_mechanism(chem_{mech} {mech})
add_executable(c_abi_contract "{root}/tests/capi/c_abi_contract.c")
set_target_properties(c_abi_contract PROPERTIES C_STANDARD 11)
target_link_libraries(c_abi_contract PRIVATE chem_{mech})
add_executable(registry_check "{root}/tests/registry/registry_check.cpp")
target_link_libraries(registry_check PRIVATE mkpp_gb300::registry)
"""


def _cmake():
    exe = shutil.which("cmake")
    if exe is None or shutil.which("gcc") is None or shutil.which("g++") is None:
        pytest.skip("cmake or the host compilers are not available")
    return exe


def _configure(tmp_path, mech):
    src, bld = tmp_path / "src", tmp_path / "build"
    src.mkdir()
    (src / "CMakeLists.txt").write_text(PROJECT.format(module=MODULE, mech=mech, root=ROOT))
    gen = ["-G", "Ninja"] if shutil.which("ninja") else []
    return subprocess.run([_cmake(), "-S", str(src), "-B", str(bld), *gen], capture_output=True, text=True,
                          timeout=300), bld


def test_cmake_project_links_mechanism_and_registry(tmp_path):
    from mkpp_gb300 import build

    cmake = _cmake()
    try:
        build.build(("chapman",))  # the build step inside CMake is then a no-op
    except RuntimeError as e:  # no nvcc
        pytest.skip(str(e))
    cfg, bld = _configure(tmp_path, "chapman")
    assert cfg.returncode == 0, cfg.stdout + cfg.stderr
    out = subprocess.run([cmake, "--build", str(bld)], capture_output=True, text=True, timeout=900)
    assert out.returncode == 0, out.stdout + out.stderr
    run = subprocess.run([str(bld / "c_abi_contract")], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and run.stdout.strip() == "ok", run.stderr
    env = {k: v for k, v in os.environ.items() if k != "MKPP_GB300_LIB_DIR"}
    reg = subprocess.run([str(bld / "registry_check"), "list"], capture_output=True, text=True, timeout=120,
                         env=env, cwd=tmp_path)
    assert reg.returncode == 0, reg.stderr
    assert "chapman" in reg.stdout.split()


def test_unknown_mechanism_stops_configure(tmp_path):
    cfg, _ = _configure(tmp_path, "no_such_mechanism")
    assert cfg.returncode != 0
    assert "FATAL ERROR: no_such_mechanism has no plan" in cfg.stderr
