"""The C++ facade (include/weldform/Domain.h) and its example driver.

CPU: the example compiles and links against the library. GPU: it runs the
reference's one-element example and agrees with the oracle (FP64, 1e-9).
"""
import os
import subprocess

import numpy as np
import pytest

from oracle import orabind as O
from weldformfem_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "weldformfem_gb300", "examples", "main_1_elem_3d.cpp")
EXE = os.path.join(ROOT, "weldformfem_gb300", "_lib", "main_1_elem_3d")


def build_example():
    lib = B.build()
    libdir = os.path.dirname(lib)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                           SRC, "-L", libdir, "-lwf_gb300", f"-Wl,-rpath,{libdir}", "-o", EXE])
    return EXE


def test_example_compiles_and_links():
    assert os.path.exists(build_example())


@pytest.mark.gpu
def test_example_matches_oracle():
    exe = build_example()
    out = subprocess.run([exe, "0"], capture_output=True, text=True, check=True).stdout
    u = np.array([[float(v) for v in ln.split()] for ln in out.strip().splitlines()])
    d = O.OracleDomain()
    d.add_box((0.1, 0.1, 0.1), 0.05)
    d.set_materials([dict(E=206e9, nu=0.3, rho=7850.0, sy0=1e10)])
    bcs = [(0, 0, 0.0), (0, 1, 0.0), (0, 2, 0.0), (1, 1, 0.0), (1, 2, 0.0), (2, 0, 0.0),
           (2, 2, 0.0), (3, 2, 0.0)] + [(i, 2, -1.0) for i in range(4, 8)]
    d.add_bcs(bcs)
    d.set_dt(0.8e-5)
    d.set_end_time(1.0e-3)
    d.init()
    assert d.solve() == 126
    uo = d.node_vec("u")
    assert np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))
