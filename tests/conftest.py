import ctypes as C
import importlib.util
import os
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
PKG_DIR = os.path.join(REPO, "boundstate-lanczos_gb300")
ORACLE_LIB = os.path.join(REPO, "oracle", "_build", "liboracle.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_package():
    if "boundstate_lanczos_gb300" in sys.modules:
        return sys.modules["boundstate_lanczos_gb300"]
    return _load("boundstate_lanczos_gb300", os.path.join(PKG_DIR, "__init__.py"))


def load_inputs():
    return _load("bsl_inputs", os.path.join(PKG_DIR, "inputs.py"))


_oracle = None


def reference_tree():
    """The reference tree the oracle recipe reads (BSL_REFERENCE_DIR or the
    recipe's default); it need not exist."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "print-ref"], capture_output=True,
                       text=True)
    return r.stdout.strip()


def load_oracle():
    """The CPU restatement (test infrastructure), built on first use."""
    global _oracle
    if _oracle is not None:
        return _oracle
    if not os.path.exists(ORACLE_LIB):
        subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "port"], check=True, capture_output=True)
    L = C.CDLL(ORACLE_LIB)
    L.orc_create.restype = C.c_void_p
    L.orc_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
    L.orc_create_synthetic.restype = C.c_void_p
    L.orc_create_synthetic.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                       C.c_char_p]
    L.orc_last_error.restype = C.c_char_p
    for f in ("orc_basis_size", "orc_vgrid_size", "orc_vblock_size"):
        getattr(L, f).restype = C.c_long
        getattr(L, f).argtypes = [C.c_void_p]
    L.orc_nn.argtypes = [C.c_void_p]
    P = C.POINTER(C.c_double)
    L.orc_hv.argtypes = [C.c_void_p, P, P, C.c_int]
    L.orc_vgrid.argtypes = [C.c_void_p, P, P]
    L.orc_vblocks.argtypes = [C.c_void_p, P]
    L.orc_destroy.argtypes = [C.c_void_p]
    L.orc_lanczos.restype = C.c_double
    L.orc_lanczos.argtypes = [C.c_void_p, C.c_int, P, P, P, P, C.c_int]
    L.orc_lancbis.argtypes = [C.c_int, P, P, P, C.c_double, C.c_double, P, P]
    L.orc_trivec.argtypes = [C.c_int, P, P, P, P, C.c_int, P]
    L.orc_ritz.argtypes = [C.c_void_p, C.c_int, P, C.c_int, P, C.c_int]
    L.orc_hf_gradient.argtypes = [C.c_void_p, C.c_int, P, P, P, P, C.c_int]
    L.orc_rigid_body_gradient.argtypes = [C.c_void_p, C.c_int, P, P, P]
    L.orc_set_charges.argtypes = [C.c_void_p, P, P, C.c_int]
    _oracle = L
    return L


def ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleModel:
    """Oracle Hamiltonian in the reference layout (CPU, FP64)."""

    def __init__(self, calculator, hv_input, extra=None, threads=8):
        self.L = load_oracle()
        h = self.L.orc_create(calculator.encode(), hv_input.encode(), extra.encode() if extra else None, threads)
        if not h:
            raise RuntimeError(self.L.orc_last_error().decode())
        self.h = C.c_void_p(h)
        self.threads = threads
        self.D = self.L.orc_basis_size(self.h)
        self.nn = self.L.orc_nn(self.h)

    def hv(self, v):
        u = np.zeros(self.D)
        self.L.orc_hv(self.h, ptr(v), ptr(u), self.threads)
        return u

    def lanczos(self, niter, v0=None):
        a, b, b2 = np.zeros(niter), np.zeros(niter + 1), np.zeros(niter + 1)
        self.L.orc_lanczos(self.h, niter, ptr(v0) if v0 is not None else None, ptr(a), ptr(b), ptr(b2),
                           self.threads)
        return a, b, b2

    def vgrid(self):
        n = self.L.orc_vgrid_size(self.h)
        a, b = np.zeros(n), np.zeros(n)
        self.L.orc_vgrid(self.h, ptr(a), ptr(b))
        return a, b

    def vblocks(self):
        out = np.zeros(self.L.orc_vblock_size(self.h))
        self.L.orc_vblocks(self.h, ptr(out))
        return out

    def hf_gradient(self, psi, natoms):
        """FP64 Hellmann-Feynman derivatives of psi[nlev, D] (continuous-grid
        Alavi SPC/E): dq[nlev, natoms], dr[nlev, natoms, 3], da[nlev, 2]."""
        ps = np.ascontiguousarray(psi, dtype=np.float64).reshape(-1, self.D)
        nlev = ps.shape[0]
        dq, dr, da = np.zeros((nlev, natoms)), np.zeros((nlev, natoms, 3)), np.zeros((nlev, 2))
        rc = self.L.orc_hf_gradient(self.h, nlev, ptr(ps), ptr(dq), ptr(dr), ptr(da), self.threads)
        if rc:
            raise RuntimeError(self.L.orc_last_error().decode())
        return dq, dr, da

    def rigid_body_gradient(self, dr):
        dr = np.ascontiguousarray(dr, dtype=np.float64)
        nlev, nmol = dr.shape[0], dr.shape[1] // 3
        dcm, dea = np.zeros((nlev, nmol, 3)), np.zeros((nlev, nmol, 3))
        if self.L.orc_rigid_body_gradient(self.h, nlev, ptr(dr), ptr(dcm), ptr(dea)):
            raise RuntimeError(self.L.orc_last_error().decode())
        return dcm, dea

    def set_charges(self, q_site=None, q_alavi=None):
        qs = None if q_site is None else np.ascontiguousarray(q_site, dtype=np.float64)
        qa = None if q_alavi is None else np.ascontiguousarray(q_alavi, dtype=np.float64)
        if self.L.orc_set_charges(self.h, None if qs is None else ptr(qs), None if qa is None else ptr(qa),
                                  self.threads):
            raise RuntimeError(self.L.orc_last_error().decode())

    def close(self):
        self.L.orc_destroy(self.h)


def oracle_lancbis(alpha, beta, beta2, emin=-10.0, emax=10.0):
    L = load_oracle()
    n = len(alpha)
    ev, er = np.zeros(n), np.zeros(n)
    ng = L.orc_lancbis(n, ptr(np.ascontiguousarray(alpha)), ptr(np.ascontiguousarray(beta)),
                       ptr(np.ascontiguousarray(beta2)), emin, emax, ptr(ev), ptr(er))
    return ev[:ng], er[:ng]


def read_boundstates(path):
    lines = open(path).read().split("\n")[4:]
    return np.array([[float(x) for x in l.split()[1:3]] for l in lines if l.strip()])


CASES = ["cage11_n10_l3_all", "seed1_n6_l3_odd", "seed0_n5_l4_even", "iso_n20_l2_all", "point_cage11_n10_l2_odd",
         "coulomb_n9_l2_all"]
# cases whose fixtures come from the compiled reference but that the CPU oracle
# restatement does not cover (other water models of the same path)
REF_ONLY_CASES = ["tip4p_seed1_n6_l3_odd", "point_tip4p_seed1_n6_l3_odd"]
# the largest potential blocks (36 and 28 functions): the oracle is pinned to
# the reference on them here, the GPU path to the oracle on the same inputs in
# test_gpu_block_sizes.py
BLOCK_CASES = ["seed1_n8_l5_all", "seed1_n8_l6_even"]


def case_info(name):
    import json
    man = json.load(open(os.path.join(GOLDEN, "manifest.json")))[name]
    d = os.path.join(GOLDEN, name)
    extra = None
    for f in ("iso_input.txt", "coulomb_input.txt"):  # the potential file the reference reads as argv[3]
        if os.path.exists(os.path.join(d, f)):
            extra = f
    return d, man, extra


@pytest.fixture
def in_case_dir(request, monkeypatch):
    def go(name):
        d, man, extra = case_info(name)
        monkeypatch.chdir(d)
        return d, man, extra
    return go
