"""Generate the committed golden fixtures from the reference itself.

Run in a container that has the reference tree (first argument, else the
BSL_REFERENCE_DIR environment variable) and
has built it with `make -C oracle ref`.  Every fixture below comes from the
UNMODIFIED reference (oracle/_ref/libref_hv.so for single Hv applications,
oracle/_ref/ref_lanczos for whole Lanczos runs) or is copied verbatim from the
reference's own stored runs (Compilation/SmallBasisTest2_*), so that the tests
can pin the oracle restatement and the GPU path where the reference tree is
absent.

    python tests/golden/make_golden.py [REFERENCE_ROOT [CASE ...]]

With case names, only those cases are (re)generated and merged into the
existing manifest.
"""
import ctypes as C
import glob
import importlib.util
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ["BSL_REFERENCE_DIR"]
ONLY = set(sys.argv[2:])
REF_LIB = os.path.join(REPO, "oracle", "_ref", "libref_hv.so")
REF_BIN = os.path.join(REPO, "oracle", "_ref", "ref_lanczos")

_spec = importlib.util.spec_from_file_location(
    "bsl_inputs", os.path.join(REPO, "boundstate-lanczos_gb300", "inputs.py"))
inputs = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(inputs)

CONTGRID = "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE"
CONTGRID_TIP4P = "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P"
ISO = "linRotCartSph_NoQuad_IsoHarmOsc"
POINT = "linRotCartSph_NoQuad_Alavi_SPCE"
POINT_TIP4P = "linRotCartSph_NoQuad_Alavi_TIP4P"
COULOMB = "linRotCartSph_NoQuad_Coulomb"

# name: (calculator, n, x_max, l_max, theta, phi, sym, geometry, niter, hv_full, iso)
# iso: the IsoHarmOsc file values, or ("coulomb", centre charge, molecule charge, ceiling),
# or ("point", universe points, universe width) for the point-grid calculators
CASES = {
    # the stored 2013-09-03 10^3 l3 runs (inputs identical to the reference's own)
    "cage11_n10_l3_all": (CONTGRID, 10, 0.4, 3, 10, 10, "All", "cage11.xyz", 300, True, None),
    # odd parity (ortho) with a synthetic cage
    "seed1_n6_l3_odd": (CONTGRID, 6, 0.08, 3, 8, 7, "Odd", "cage_seed1.xyz", 200, True, None),
    # even parity (para) with the CPU-workload angular grid
    "seed0_n5_l4_even": (CONTGRID, 5, 0.08, 4, 12, 12, "Even", "cage_seed0.xyz", 200, True, None),
    # isotropic harmonic oscillator (analytic check), orientation independent
    "iso_n20_l2_all": (ISO, 20, 0.3, 2, 4, 4, "All", "NULL", 300, True, (2.015650064, 24.1, 100.0)),
    # the CPU workload itself: 15^3 even l<=4 12 x 24, cage seed 0, 600 iterations
    "cpu_workload": (CONTGRID, 15, 0.08, 4, 12, 12, "Even", "cage_seed0.xyz", 600, False, None),
    # the same continuous-grid path with TIP4P water
    "tip4p_seed1_n6_l3_odd": (CONTGRID_TIP4P, 6, 0.08, 3, 8, 7, "Odd", "cage_seed1.xyz", 200, True, None),
    # point-grid Alavi SPC/E with the inputs of the reference's stored 2013-08-30 15:06 run
    "point_cage11_n10_l2_odd": (POINT, 10, 0.4, 2, 10, 10, "Odd", "cage11.xyz", 300, True, ("point", 20, 0.48)),
    # point-grid Alavi TIP4P, universe finer than the basis grid
    "point_tip4p_seed1_n6_l3_odd": (POINT_TIP4P, 6, 0.08, 3, 8, 7, "Odd", "cage_seed1.xyz", 200, True,
                                    ("point", 13, 0.1)),
    # charge at the origin (an odd grid has a point there: 1/0 is clipped)
    "coulomb_n9_l2_all": (COULOMB, 9, 0.3, 2, 4, 4, "All", "NULL", 300, True, ("coulomb", 0.1, -0.1, -20.0)),
    # the largest blocks of the potential stream: 36 functions (all l <= 5) and
    # 28 (even l <= 6), the inputs of the GPU block-size tests
    "seed1_n8_l5_all": (CONTGRID, 8, 0.08, 5, 8, 8, "All", "cage_seed1.xyz", 200, True, None),
    "seed1_n8_l6_even": (CONTGRID, 8, 0.08, 6, 8, 8, "Even", "cage_seed1.xyz", 200, True, None),
}


def ref_hv(calc, hv_path, extra):
    lib = C.CDLL(REF_LIB)
    lib.ref_hv_setup.restype = C.c_long
    D = lib.ref_hv_setup(calc.encode(), hv_path.encode(), extra.encode() if extra else None)
    P = C.POINTER(C.c_double)
    rng = np.random.default_rng(20131903)
    v = rng.standard_normal(D)
    u = np.zeros(D)
    lib.ref_hv(v.ctypes.data_as(P), u.ctypes.data_as(P))
    return D, u


def run_ref_lanczos(case_dir, calc, extra):
    tmp = tempfile.mkdtemp()
    for f in os.listdir(case_dir):
        shutil.copy(os.path.join(case_dir, f), tmp)
    lz = os.path.join(tmp, "lanczos_input.txt")
    txt = open(lz).read().replace("OutputDirectoryPath= ./", "OutputDirectoryPath= %s/out_" % tmp)
    open(lz, "w").write(txt)
    args = [REF_BIN, "lanczos_input.txt", "hv_input.txt"] + ([extra] if extra else [])
    log = subprocess.run(args, cwd=tmp, capture_output=True, text=True, check=True).stdout
    ab = [l.split() for l in log.splitlines() if re.match(r"^\d+ \S+ \S+$", l)]
    alpha = np.array([float(x[1]) for x in ab])
    beta = np.array([float(x[2]) for x in ab])
    bs = glob.glob(os.path.join(tmp, "out_*", "boundstates.txt"))[0]
    shutil.copy(bs, os.path.join(case_dir, "ref_boundstates.txt"))
    shutil.rmtree(tmp)
    return alpha, beta


# Fixture pinning the FP64 Hellmann-Feynman oracle: for a fixed vector psi the
# Rayleigh quotient E = psi.H psi / psi.psi of the reference's own H has
# dE/dtheta = psi.(dH/dtheta) psi / psi.psi exactly, so central differences of
# E through the compiled reference, with the cage's centres and Euler angles
# moved in the .xyz it reads, check the oracle's site derivatives and its
# chain rule to the rigid-body coordinates.
HF_FD_CASE = "hf_fd_seed1_n5_l3_odd"
HF_FD_STEP = 1e-5
HF_FD_PARAMS = [("cm", 0, 0), ("cm", 3, 1), ("cm", 11, 2), ("cm", 17, 0), ("euler", 2, 0), ("euler", 5, 1),
                ("euler", 9, 2), ("euler", 14, 0), ("euler", 19, 1)]


def make_hf_fd():
    d = os.path.join(HERE, HF_FD_CASE)
    os.makedirs(d, exist_ok=True)
    waters = inputs.dodecahedral_cage(1)
    inputs.write_cage_xyz(os.path.join(d, "cage.xyz"), waters)
    inputs.write_hv_input(os.path.join(d, "hv_input.txt"),
                          inputs.hv_fields(5, 0.08, 3, 6, 5, "cage.xyz", HF_FD_CASE, "Odd"))
    lib = C.CDLL(REF_LIB)
    lib.ref_hv_setup.restype = C.c_long
    P = C.POINTER(C.c_double)
    cwd = os.getcwd()
    os.chdir(d)
    try:
        D = lib.ref_hv_setup(CONTGRID.encode(), b"hv_input.txt", None)
        lmax, N = 3, 125
        ls = [l for m in range(-lmax, lmax + 1) for l in range(abs(m), lmax + 1)]
        psi = np.random.default_rng(7).standard_normal(D)
        for n, l in enumerate(ls):
            if l % 2 == 0:
                psi[n * N:(n + 1) * N] = 0.0  # outside the odd block

        def energy(ws):
            inputs.write_cage_xyz("cage_fd.xyz", ws)
            inputs.write_hv_input("hv_fd.txt", inputs.hv_fields(5, 0.08, 3, 6, 5, "cage_fd.xyz", HF_FD_CASE, "Odd"))
            lib.ref_hv_setup(CONTGRID.encode(), b"hv_fd.txt", None)
            u = np.zeros(D)
            lib.ref_hv(psi.ctypes.data_as(P), u.ctypes.data_as(P))
            return float(psi @ u / (psi @ psi))

        rows = []
        for kind, m, k in HF_FD_PARAMS:
            e = []
            for sgn in (1.0, -1.0):
                ws = [(nm, list(cm), list(ea)) for nm, cm, ea in waters]
                (ws[m][1] if kind == "cm" else ws[m][2])[k] += sgn * HF_FD_STEP
                e.append(energy(ws))
            rows.append([e[0], e[1]])
        for f in ("cage_fd.xyz", "hv_fd.txt"):
            os.remove(f)
    finally:
        os.chdir(cwd)
    np.savez(os.path.join(d, "ref_rayleigh_fd.npz"), psi=psi, e_pm=np.array(rows), step=HF_FD_STEP,
             params=np.array([[0 if kind == "cm" else 1, m, k] for kind, m, k in HF_FD_PARAMS]))
    print(HF_FD_CASE, np.array(rows)[:, 0] - np.array(rows)[:, 1])


def main():
    if ONLY == {HF_FD_CASE}:
        make_hf_fd()
        return
    shutil.copy(os.path.join(REF, "Compilation", "sII_smallCage11_CM_EA_ZYZ.xyz"), os.path.join(HERE, "cage11.xyz"))
    for seed in (0, 1):
        inputs.write_cage_xyz(os.path.join(HERE, "cage_seed%d.xyz" % seed), inputs.dodecahedral_cage(seed))
    manifest = {}
    if ONLY:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)
    for name, (calc, n, xm, lmax, th, ph, sym, geo, niter, full, iso) in CASES.items():
        if ONLY and name not in ONLY:
            continue
        d = os.path.join(HERE, name)
        os.makedirs(d, exist_ok=True)
        if geo != "NULL":
            shutil.copy(os.path.join(HERE, geo), os.path.join(d, geo))
        point = iso[1:] if iso and iso[0] == "point" else None
        if name.startswith("cage11") or name == "point_cage11_n10_l2_odd":
            vals = inputs.hv_fields(n, xm, lmax, th, ph, geo, "SmallBasisTest2", sym, rot_const=0.7096487130193394,
                                    point_grid=point)
        else:
            vals = inputs.hv_fields(n, xm, lmax, th, ph, geo, name, sym, point_grid=point)
        if calc == ISO:
            vals[16] = 0.709652722117881
            vals[19] = 100.0
        inputs.write_hv_input(os.path.join(d, "hv_input.txt"), vals)
        inputs.write_lanczos_input(os.path.join(d, "lanczos_input.txt"), niter, calc)
        extra = None
        if calc == ISO:
            inputs.write_isoharmosc_input(os.path.join(d, "iso_input.txt"), *iso)
            extra = "iso_input.txt"
        elif calc == COULOMB:
            inputs.write_coulomb_input(os.path.join(d, "coulomb_input.txt"), *iso[1:])
            extra = "coulomb_input.txt"
        cwd = os.getcwd()
        os.chdir(d)
        try:
            D, u = ref_hv(calc, "hv_input.txt", extra)
        finally:
            os.chdir(cwd)
        rec = {"calculator": calc, "basis_size": int(D), "niter": niter, "hv_seed": 20131903,
               "hv_norm": float(np.linalg.norm(u)), "hv_sum": float(u.sum())}
        if full:
            np.save(os.path.join(d, "ref_hv.npy"), u)
        else:
            idx = np.arange(0, D, max(1, D // 4096))
            np.savez(os.path.join(d, "ref_hv_sample.npz"), idx=idx, val=u[idx])
        alpha, beta = run_ref_lanczos(d, calc, extra)
        np.savez(os.path.join(d, "ref_alpha_beta.npz"), alpha=alpha, beta=beta)
        manifest[name] = rec
        print(name, rec)
    if ONLY:
        with open(os.path.join(HERE, "manifest.json"), "w") as f:
            json.dump(manifest, f, indent=1)
        return
    # the reference's own stored 2013 runs that the final tree reproduces
    stored = {}
    for run in ("SmallBasisTest2_2013-09-03_18_36_00", "SmallBasisTest2_2013-09-03_19_06_47",
                "SmallBasisTest2_2013-08-30_15_06_49"):
        lines = open(os.path.join(REF, "Compilation", run, "boundstates.txt")).read().split("\n")[4:]
        vals = [[float(x) for x in l.split()[1:3]] for l in lines if l.strip()]
        niter = int(re.search(r"numberOfIterations= (\d+)",
                              open(os.path.join(REF, "Compilation", run,
                                                "LanczosInputFileTobySmallBasisTest2.txt")).read()).group(1))
        stored[run] = {"niter": niter, "levels": vals}
    with open(os.path.join(HERE, "stored_2013_runs.json"), "w") as f:
        json.dump(stored, f, indent=0)
    make_hf_fd()
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
