"""The CMake package (CMakeLists.txt, cmake/): installed with the library
that build.py made, a consumer project of the reference's shape --
find_package(BSplineInterpolation 2) and target_link_libraries(app
BSplineInterpolation) -- configures, compiles against the drop-in headers
(#include "Interpolation.hpp", as the reference's own tests do) and links the
CUDA library. Running the consumer needs a GPU and is the C++ drop-in test's
job; this test stops at the link. Skipped where cmake is absent."""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CONSUMER_CMAKE = """cmake_minimum_required(VERSION 3.18)
project(consumer LANGUAGES CXX)
find_package(BSplineInterpolation 2 REQUIRED)
add_executable(app app.cpp)
target_link_libraries(app BSplineInterpolation)
"""

CONSUMER_SRC = """#include "Interpolation.hpp"
#include <iostream>
int main() {
    intp::Mesh<double, 2> mesh(8, 9);
    for (std::size_t i = 0; i < 8; ++i)
        for (std::size_t j = 0; j < 9; ++j) mesh(i, j) = 0.1 * i + 0.01 * j;
    intp::InterpolationFunction<double, 2, 3> f(mesh, std::make_pair(0.0, 1.0), std::make_pair(0.0, 2.0));
    std::cout << f(0.5, 1.0) << std::endl;
    return 0;
}
"""


def _run(cmd, cwd):
    r = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cmake_package_install_and_consumer(tmp_path):
    cmake = shutil.which("cmake")
    if cmake is None or shutil.which("g++") is None:
        pytest.skip("cmake or a host compiler is absent")
    from bsplineinterpolation_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    prefix = tmp_path / "prefix"
    _run([cmake, "-S", REPO, "-B", str(tmp_path / "pkg"), "-DINTP_GB300_PREBUILT=" + _lib.LIB_PATH,
          "-DCMAKE_INSTALL_PREFIX=" + str(prefix)], REPO)
    _run([cmake, "--install", str(tmp_path / "pkg")], REPO)
    assert (prefix / "include" / "BSplineInterpolation" / "Interpolation.hpp").exists()
    assert (prefix / "include" / "intp_gpu.h").exists()
    cons = tmp_path / "consumer"
    cons.mkdir()
    (cons / "CMakeLists.txt").write_text(CONSUMER_CMAKE)
    (cons / "app.cpp").write_text(CONSUMER_SRC)
    _run([cmake, "-S", str(cons), "-B", str(cons / "build"), "-DCMAKE_PREFIX_PATH=" + str(prefix)], REPO)
    _run([cmake, "--build", str(cons / "build")], REPO)
    assert (cons / "build" / "app").exists()
