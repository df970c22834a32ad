"""Drop-in checks: the reference-shaped C++ classes (include/acogpu_colony.hpp)
behave like the Python binding, and the reference's own driver compiles and
links against them unchanged."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import acogpu_gb300 as aco
import oracle
from acogpu_gb300.colony import LIB_PATH
from helpers import instance

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = oracle.REF_SOURCES


def _compiler():
    return shutil.which("g++")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")) or not shutil.which("nvcc"),
                    reason="reference sources or nvcc absent")
def test_reference_driver_links_against_the_shim(tmp_path):
    """src/Setup.cpp + src/TSP.cpp + the reference's CLI, writer, reader and
    timer, unmodified, built against include/reference_shim and
    libacogpu.so instead of src/Colony.cu and src/AntSystem.cu."""
    aco.lib()
    src = os.path.join(REF, "src")
    files = [os.path.join(src, f) for f in ("Setup.cpp", "TSP.cpp", "Writer.cpp",
                                            "Commandline.cpp", "Timer.cpp", "TSPReader.cu",
                                            "Utils.cu")]
    out = tmp_path / "acouav_gb300"
    cmd = ["nvcc", "-O1", "-w", "-I" + os.path.join(ROOT, "include", "reference_shim"),
           "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REF, "inc", "gpu"),
           "-I" + os.path.join(REF, "inc", "noaging"), "-I" + os.path.join(REF, "inc", "nobroker"),
           "-I" + os.path.join(REF, "inc"), "-x", "cu", *files,
           "-L" + os.path.dirname(LIB_PATH), "-lacogpu", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert out.exists()


def _build_driver(tmp_path):
    aco.lib()
    exe = tmp_path / "shim_driver"
    cmd = [_compiler(), "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "shim_driver.cpp"),
           "-L" + os.path.dirname(LIB_PATH), "-lacogpu",
           "-Wl,-rpath," + os.path.dirname(LIB_PATH), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


@pytest.mark.skipif(_compiler() is None, reason="no C++ compiler")
def test_shim_compiles(tmp_path):
    _build_driver(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("aging", [0, 1])
def test_cpp_shim_matches_python_binding(tmp_path, aging):
    exe = _build_driver(tmp_path)
    _, _, d = instance(60, 17)
    path = tmp_path / "dist.bin"
    d.astype(np.int32).tofile(path)
    m, iters = 24, 12
    r = subprocess.run([str(exe), str(path), "60", str(m), str(iters), str(aging)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines() if " " in l)
    if aging:
        py = aco.AntSystem(d, 60, m, 1.0, 2.0, 0.5, 3, 5, 10, 2, m // 2, 100)
    else:
        py = aco.AntSystem(d, 60, m, 1.0, 2.0, 0.5)
    py.initialize()
    for _ in range(iters):
        py.constructSolution()
    assert int(lines["best"]) == py.getGlobBestDist()
    assert lines["tour"] == py.getTour()
    assert lines["name"] == "Ant System"
