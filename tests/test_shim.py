"""The reference-signature shim (include/bsl_reference_shim.h), used the way
the reference's driver uses its registry: tests/shim_driver.cpp links the
library, looks a `_GB300` HvCalculator up, runs HvPrep once and Hv on a
seeded vector.  On the CPU: the driver builds and links, and the shim header
compiles after the reference's own lanczosStor/generalStor definitions
(where the reference tree is present).  On the GPU: uec += H vec through the
shim equals the reference's own H v (<= 1e-10 relative)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, REPO, case_info, reference_tree

INCLUDE = os.path.join(REPO, "include")
DRIVER = os.path.join(REPO, "tests", "shim_driver.cpp")
REF_TREE = reference_tree()


def build_driver(out_dir):
    exe = os.path.join(out_dir, "shim_driver")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", INCLUDE, DRIVER, "-o", exe, "-L", PKG_DIR, "-lbsl_gb300",
                    "-Wl,-rpath," + PKG_DIR], check=True, capture_output=True, text=True)
    return exe


def test_shim_driver_builds_against_the_library(tmp_path):
    exe = build_driver(str(tmp_path))
    p = subprocess.run([exe], capture_output=True, text=True)
    assert p.returncode == 2 and "usage" in p.stderr


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_TREE, "headLoop")), reason="reference tree absent")
def test_shim_header_accepts_the_reference_containers(tmp_path):
    src = tmp_path / "with_reference_containers.cpp"
    src.write_text('#include "interfaceContainers.h"\n#include "bsl_reference_shim.h"\n'
                   "int main() { lanczosStor l; l.total_basis_size = 1; l.sim_descr = \"x\";\n"
                   "  generalStor* g = bsl_reference_storage(\"linRotCartSph_NoQuad_Coulomb_GB300\");\n"
                   "  return g == nullptr; }\n")
    cb = os.path.join(REF_TREE, "Hv-calculators", "linRotor", "cartSphBasis")
    inc = [os.path.join(REF_TREE, "headLoop", "InterfaceCode"), os.path.join(cb, "librarySources", "matVecClasses"),
           os.path.join(cb, "librarySources", "general"), INCLUDE]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w", "-DLINUX"] + sum([["-I", d] for d in inc], []) + [str(src)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["seed1_n6_l3_odd", "iso_n20_l2_all", "coulomb_n9_l2_all"])
def test_shim_hv_matches_reference(tmp_path, name):
    d, man, extra = case_info(name)
    exe = build_driver(str(tmp_path))
    v = np.random.default_rng(man["hv_seed"]).standard_normal(man["basis_size"])
    vin, uout = str(tmp_path / "vec.bin"), str(tmp_path / "uec.bin")
    v.tofile(vin)
    env = dict(os.environ)
    env.pop("BSL_PRECISION", None)  # FP64
    p = subprocess.run([exe, man["calculator"] + "_GB300", "hv_input.txt", extra or "-", vin, uout], cwd=d,
                       capture_output=True, text=True, env=env, timeout=600)
    assert p.returncode == 0, p.stderr[-3000:]
    size = int(p.stdout.strip().splitlines()[-1].split("|")[0])
    assert size == man["basis_size"]
    u = np.fromfile(uout)
    ref = np.load(os.path.join(d, "ref_hv.npy"))
    assert np.max(np.abs(u - ref)) / np.max(np.abs(ref)) <= 1e-10
