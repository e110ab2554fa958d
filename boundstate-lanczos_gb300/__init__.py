"""Python mirror of the reference's HvCalculator plugin interface over the C ABI.

The reference registers an HvCalculator by name and hands its Lanczos driver
an (HvPrep, Hv) function-pointer pair plus opaque storage
(headLoop/InterfaceCode/interface.cpp:3-250).  `hv_interface_setup(name)`
returns the same pair for the GB300 calculators, bound to libbsl_gb300.so
through ctypes; `Hamiltonian` exposes the device-resident extras (the Lanczos
loop on the GPU, packed-layout applications, Ritz vectors).

The library must have been built (build.py); there is no CPU fallback: a
missing library raises immediately.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbsl_gb300.so")

OK, ERR_INPUT, ERR_CUDA, ERR_STATE, ERR_BREAKDOWN, ERR_UNSUPPORTED, ERR_NOMEM = range(7)
SYM = {"All": 0, "Even": 1, "Odd": 2}
POT_ALAVI_SPCE, POT_ISOHARMOSC, POT_ALAVI_TIP4P = 0, 1, 2
POT_POINT_ALAVI_SPCE, POT_POINT_ALAVI_TIP4P, POT_COULOMB = 3, 4, 5
PREC = {"fp64": 0, "mixed": 1}
START = {"uniform": 0, "normal": 1}
KINETIC = {"simt": 0, "tensor": 1}
VFORMAT = {"fp32": 0, "bf16": 1, "gaunt": 2}
MIXED_UNIT_ROUNDOFF = 4.0e-15  # BSL_MIXED_UNIT_ROUNDOFF
MIXED_REL_NOISE = 1.0e-9  # BSL_MIXED_REL_NOISE
CALCULATORS = {
    "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE": POT_ALAVI_SPCE,
    "linRotCartSph_NoQuad_IsoHarmOsc": POT_ISOHARMOSC,
    "linRotCartSph_NoQuad_ContGrid_Alavi_SPCE_GB300": POT_ALAVI_SPCE,
    "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P": POT_ALAVI_TIP4P,
    "linRotCartSph_NoQuad_ContGrid_Alavi_TIP4P_GB300": POT_ALAVI_TIP4P,
    "linRotCartSph_NoQuad_IsoHarmOsc_GB300": POT_ISOHARMOSC,
    "linRotCartSph_NoQuad_Alavi_SPCE": POT_POINT_ALAVI_SPCE,
    "linRotCartSph_NoQuad_Alavi_SPCE_GB300": POT_POINT_ALAVI_SPCE,
    "linRotCartSph_NoQuad_Alavi_TIP4P": POT_POINT_ALAVI_TIP4P,
    "linRotCartSph_NoQuad_Alavi_TIP4P_GB300": POT_POINT_ALAVI_TIP4P,
    "linRotCartSph_NoQuad_Coulomb": POT_COULOMB,
    "linRotCartSph_NoQuad_Coulomb_GB300": POT_COULOMB,
}


class BslError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("bsl error %d: %s" % (code, msg))
        self.code = code


class HvParams(C.Structure):
    """Mirror of bsl_hv_params (include/bsl.h)."""
    _fields_ = [("nx", C.c_int), ("x_max", C.c_double), ("ny", C.c_int), ("y_max", C.c_double),
                ("nz", C.c_int), ("z_max", C.c_double), ("l_max", C.c_int), ("theta_points", C.c_int),
                ("phi_points", C.c_int), ("pnx", C.c_int), ("px_max", C.c_double), ("pny", C.c_int),
                ("py_max", C.c_double), ("pnz", C.c_int), ("pz_max", C.c_double), ("total_mass", C.c_double),
                ("rotational_constant", C.c_double), ("geometry_filename", C.c_char * 1024),
                ("simulation_title", C.c_char * 256), ("ceiling_potential", C.c_double),
                ("quadrature_study", C.c_int), ("symmetry", C.c_int), ("potential", C.c_int),
                ("iso_mass", C.c_double), ("iso_frequency", C.c_double), ("iso_ceiling", C.c_double),
                ("precision", C.c_int), ("device", C.c_int), ("keep_potential_grid", C.c_int),
                ("coulomb_centre_charge", C.c_double), ("coulomb_mol_charge", C.c_double),
                ("coulomb_ceiling", C.c_double)]


_lib = None
_P = C.POINTER(C.c_double)


def lib():
    """Load libbsl_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libbsl_gb300.so is not built: run boundstate-lanczos_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    L.bsl_last_error.restype = C.c_char_p
    L.bsl_basis_size.restype = C.c_longlong
    L.bsl_packed_size.restype = C.c_longlong
    L.bsl_vgrid_size.restype = C.c_longlong
    L.bsl_vblock_size.restype = C.c_longlong
    L.bsl_stream.restype = C.c_void_p
    L.bsl_hv_prep.argtypes = [C.POINTER(HvParams), C.POINTER(C.c_void_p)]
    for name in ("bsl_basis_size", "bsl_packed_size", "bsl_packed_nn", "bsl_vgrid_size", "bsl_vblock_size",
                 "bsl_stream", "bsl_destroy"):
        getattr(L, name).argtypes = [C.c_void_p]
    L.bsl_hv_apply.argtypes = [C.c_void_p, _P, _P]
    L.bsl_hv_apply_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.bsl_set_precision.argtypes = [C.c_void_p, C.c_int]
    L.bsl_set_kinetic_engine.argtypes = [C.c_void_p, C.c_int]
    L.bsl_kinetic_engine.argtypes = [C.c_void_p]
    L.bsl_lanczos_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_ulonglong, _P, _P, _P]
    L.bsl_lanczos_run_batch.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_ulonglong,
                                        C.POINTER(_P), C.POINTER(_P), C.POINTER(_P)]
    L.bsl_lanczos_run_batch_streams.argtypes = L.bsl_lanczos_run_batch.argtypes
    L.bsl_lanczos_step_host.argtypes = [C.c_void_p, _P, _P, _P, _P, _P]
    L.bsl_good_eigenvalues.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, _P, _P, C.POINTER(C.c_int)]
    L.bsl_good_eigenvalues_unit.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_double, _P, _P,
                                            C.POINTER(C.c_int)]
    L.bsl_good_eigenvalues_noise.argtypes = [C.c_int, _P, _P, _P, C.c_double, C.c_double, C.c_double, C.c_double,
                                             _P, _P, C.POINTER(C.c_int)]
    L.bsl_write_boundstates.argtypes = [C.c_char_p, C.c_char_p, C.c_int, _P, _P]
    L.bsl_write_tm_vectors.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int, _P]
    L.bsl_write_ritz_vectors.argtypes = [C.c_char_p, C.c_char_p, C.c_longlong, C.c_int, _P]
    L.bsl_ritz_vectors_start.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_ulonglong, _P, C.c_int, _P]
    L.bsl_hv_prep_cage.argtypes = [C.POINTER(HvParams), C.c_int, _P, _P, _P, _P, C.POINTER(C.c_void_p)]
    L.bsl_hf_gradient.argtypes = [C.c_void_p, C.c_int, _P, _P, _P, _P]
    L.bsl_rigid_body_gradient.argtypes = [C.c_int, C.c_int, _P, _P, C.c_int, _P, _P, _P]
    L.bsl_cage_sites.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P]
    L.bsl_tm_eigenvectors.argtypes = [C.c_int, _P, _P, _P, _P, C.c_int, _P]
    L.bsl_ritz_vectors.argtypes = [C.c_void_p, C.c_int, _P, C.c_int, _P]
    L.bsl_last_run_ms_per_iter.argtypes = [C.c_void_p, _P]
    L.bsl_copy_vgrid.argtypes = [C.c_void_p, _P, _P]
    L.bsl_copy_vblocks.argtypes = [C.c_void_p, _P]
    L.bsl_parse_hv_input.argtypes = [C.c_char_p, C.POINTER(HvParams)]
    L.bsl_parse_isoharmosc_input.argtypes = [C.c_char_p, C.POINTER(HvParams)]
    L.bsl_parse_coulomb_input.argtypes = [C.c_char_p, C.POINTER(HvParams)]
    L.bsl_calculator_potential.argtypes = [C.c_char_p, C.POINTER(C.c_int)]
    L.bsl_debug_inject_timeout.argtypes = [C.c_void_p, C.c_int]
    L.bsl_autotune.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                               _P]
    L.bsl_set_kinetic_slices.argtypes = [C.c_void_p, C.c_int]
    L.bsl_set_potential_format.argtypes = [C.c_void_p, C.c_int]
    L.bsl_potential_format.argtypes = [C.c_void_p]
    L.bsl_gaunt_residual.argtypes = [C.c_void_p]
    L.bsl_gaunt_residual.restype = C.c_double
    _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise BslError(rc, lib().bsl_last_error().decode())


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def parse_hv_input(path):
    p = HvParams()
    _check(lib().bsl_parse_hv_input(path.encode(), C.byref(p)))
    return p


def good_eigenvalues(alpha, beta, beta2, emin=-10.0, emax=10.0, unit_roundoff=None, rel_noise=None):
    """Cullum-Willoughby good eigenvalues in (emin, emax] and error estimates.

    unit_roundoff: None for the reference's FP64 tolerances, else the unit
    roundoff the multiplicity tolerances are built on (bsl_good_eigenvalues_unit);
    rel_noise: a floor under the multiplicity window relative to max|T|
    (bsl_good_eigenvalues_noise).  For runs of the mixed path pass
    unit_roundoff=MIXED_UNIT_ROUNDOFF, rel_noise=MIXED_REL_NOISE."""
    alpha, beta, beta2 = (np.ascontiguousarray(x, dtype=np.float64) for x in (alpha, beta, beta2))
    niter = len(alpha)
    ev = np.zeros(niter)
    er = np.zeros(niter)
    ng = C.c_int(0)
    if rel_noise is not None:
        unit = unit_roundoff if unit_roundoff is not None else 2.0 ** -52
        _check(lib().bsl_good_eigenvalues_noise(niter, _ptr(alpha), _ptr(beta), _ptr(beta2), emin, emax, unit,
                                                rel_noise, _ptr(ev), _ptr(er), C.byref(ng)))
    elif unit_roundoff is None:
        _check(lib().bsl_good_eigenvalues(niter, _ptr(alpha), _ptr(beta), _ptr(beta2), emin, emax, _ptr(ev),
                                          _ptr(er), C.byref(ng)))
    else:
        _check(lib().bsl_good_eigenvalues_unit(niter, _ptr(alpha), _ptr(beta), _ptr(beta2), emin, emax,
                                               unit_roundoff, _ptr(ev), _ptr(er), C.byref(ng)))
    return ev[:ng.value].copy(), er[:ng.value].copy()


def tm_eigenvectors(alpha, beta, beta2, evals):
    alpha, beta, beta2, evals = (np.ascontiguousarray(x, dtype=np.float64) for x in (alpha, beta, beta2, evals))
    niter, ngood = len(alpha), len(evals)
    out = np.zeros(niter * ngood)
    _check(lib().bsl_tm_eigenvectors(niter, _ptr(alpha), _ptr(beta), _ptr(beta2), _ptr(evals), ngood, _ptr(out)))
    return out.reshape(ngood, niter)  # row n = column n of the column-major evtr


def lanczos_batch(hamiltonians, niter, start="uniform", seed=0, grouped=True):
    """Loop 1 for several prepared problems at once: grouped launches where the
    problems allow them (bsl_lanczos_run_batch), or with grouped=False one
    stream per problem (bsl_lanczos_run_batch_streams); returns a list of
    (alpha, beta, beta2)."""
    n = len(hamiltonians)
    out = [(np.zeros(niter), np.zeros(niter + 1), np.zeros(niter + 1)) for _ in range(n)]
    hs = (C.c_void_p * n)(*[h.handle for h in hamiltonians])
    arr = [(_P * n)(*[_ptr(o[k]) for o in out]) for k in range(3)]
    f = lib().bsl_lanczos_run_batch if grouped else lib().bsl_lanczos_run_batch_streams
    _check(f(hs, n, niter, START[start], seed, arr[0], arr[1], arr[2]))
    return out


def autotune(hamiltonians, iters=200):
    """Pick the launch shapes of one problem or a batch by timing
    (bsl_autotune); returns (potential-stream CTAs per SM, update CTAs per SM,
    best ms per iteration)."""
    n = len(hamiltonians)
    hs = (C.c_void_p * n)(*[h.handle for h in hamiltonians])
    vs, up, ms = C.c_int(0), C.c_int(0), np.zeros(1)
    _check(lib().bsl_autotune(hs, n, iters, C.byref(vs), C.byref(up), _ptr(ms)))
    return vs.value, up.value, float(ms[0])


def _f64(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def sites_per_molecule(potential):
    return 4 if potential in (POT_ALAVI_TIP4P, POT_POINT_ALAVI_TIP4P) else 3


def cage_sites(cm_ang, euler, q_site=None, potential=POT_ALAVI_SPCE):
    """Site positions (nm, [S nmol, 3]) and charges of rigid SPC/E (S = 3) or TIP4P (S = 4) waters."""
    cm, ea = _f64(cm_ang).reshape(-1, 3), _f64(euler).reshape(-1, 3)
    n, S = cm.shape[0], sites_per_molecule(potential)
    xyz, q = np.zeros((S * n, 3)), np.zeros(S * n)
    qs = None if q_site is None else _f64(q_site)
    _check(lib().bsl_cage_sites(potential, n, _ptr(cm), _ptr(ea), None if qs is None else _ptr(qs), _ptr(xyz),
                                _ptr(q)))
    return xyz, q


def rigid_body_gradient(cm_ang, euler, dr_site, potential=POT_ALAVI_SPCE):
    """Chain rule dE/dr_site [nlev, S nmol, 3] -> (dE/dcm [nlev, nmol, 3] per Angstrom, dE/deuler)."""
    cm, ea = _f64(cm_ang).reshape(-1, 3), _f64(euler).reshape(-1, 3)
    n, S = cm.shape[0], sites_per_molecule(potential)
    dr = _f64(dr_site).reshape(-1, S * n, 3)
    nlev = dr.shape[0]
    dcm, dea = np.zeros((nlev, n, 3)), np.zeros((nlev, n, 3))
    _check(lib().bsl_rigid_body_gradient(potential, n, _ptr(cm), _ptr(ea), nlev, _ptr(dr), _ptr(dcm), _ptr(dea)))
    return dcm, dea


def write_boundstates(directory, sim_descr, evals, errs):
    """boundstates.txt and states_zpe.txt in the reference's format."""
    evals, errs = (np.ascontiguousarray(x, dtype=np.float64) for x in (evals, errs))
    _check(lib().bsl_write_boundstates(directory.encode(), sim_descr.encode(), len(evals), _ptr(evals), _ptr(errs)))


def write_tm_vectors(directory, sim_descr, evtr_rows):
    """lv: squared Tm eigenvector coefficients (rows as from tm_eigenvectors)."""
    rows = np.ascontiguousarray(evtr_rows, dtype=np.float64)
    ngood, niter = rows.shape
    _check(lib().bsl_write_tm_vectors(directory.encode(), sim_descr.encode(), niter, ngood, _ptr(rows.reshape(-1))))


def write_ritz_vectors(directory, sim_descr, ritz):
    """eigVecFile.txt: Ritz vectors (ngood x basis_size) in the reference layout."""
    r = np.ascontiguousarray(ritz, dtype=np.float64)
    ngood, size = r.shape
    _check(lib().bsl_write_ritz_vectors(directory.encode(), sim_descr.encode(), size, ngood, _ptr(r.reshape(-1))))


class Hamiltonian:
    """A prepared H on one GPU (the reference's HvPrep result)."""

    def __init__(self, hv_input, calculator="linRotCartSph_NoQuad_ContGrid_Alavi_SPCE", extra_input=None,
                 precision="fp64", device=0, params=None):
        L = lib()
        p = params if params is not None else parse_hv_input(hv_input)
        pot = C.c_int(0)
        _check(L.bsl_calculator_potential(calculator.encode(), C.byref(pot)))
        p.potential = pot.value
        if p.potential == POT_ISOHARMOSC:
            _check(L.bsl_parse_isoharmosc_input(extra_input.encode(), C.byref(p)))
        if p.potential == POT_COULOMB:
            _check(L.bsl_parse_coulomb_input(extra_input.encode(), C.byref(p)))
        p.precision = PREC[precision]
        p.device = device
        self.params = p
        h = C.c_void_p()
        _check(L.bsl_hv_prep(C.byref(p), C.byref(h)))
        self._h = h
        self.basis_size = L.bsl_basis_size(h)
        self.packed_size = L.bsl_packed_size(h)
        self.nn = L.bsl_packed_nn(h)

    @classmethod
    def from_cage(cls, params, cm_ang, euler, q_site=None, q_alavi=None, precision="fp64", device=0,
                  keep_potential_grid=True, potential=POT_ALAVI_SPCE):
        """HvPrep for an Alavi SPC/E or TIP4P cage given as arrays (bsl_hv_prep_cage)."""
        self = cls.__new__(cls)
        L = lib()
        p = HvParams()
        C.pointer(p)[0] = params
        p.potential = potential
        p.precision = PREC[precision]
        p.device = device
        p.keep_potential_grid = 1 if keep_potential_grid else 0
        cm, ea = _f64(cm_ang).reshape(-1), _f64(euler).reshape(-1)
        qs = None if q_site is None else _f64(q_site)
        qa = None if q_alavi is None else _f64(q_alavi)
        h = C.c_void_p()
        self._h = None
        _check(L.bsl_hv_prep_cage(C.byref(p), len(cm) // 3, _ptr(cm), _ptr(ea), None if qs is None else _ptr(qs),
                                  None if qa is None else _ptr(qa), C.byref(h)))
        self.params = p
        self._h = h
        self.basis_size = L.bsl_basis_size(h)
        self.packed_size = L.bsl_packed_size(h)
        self.nn = L.bsl_packed_nn(h)
        return self

    def hf_gradient(self, psi, natoms):
        """Hellmann-Feynman derivatives of the levels of eigenvectors psi [nlev, basis_size]:
        (dE/dq_site [nlev, natoms], dE/dr_site [nlev, natoms, 3], dE/dq_alavi [nlev, 2])."""
        ps = _f64(psi).reshape(-1, self.basis_size)
        nlev = ps.shape[0]
        dq, dr, da = np.zeros((nlev, natoms)), np.zeros((nlev, natoms, 3)), np.zeros((nlev, 2))
        _check(lib().bsl_hf_gradient(self._h, nlev, _ptr(ps), _ptr(dq), _ptr(dr), _ptr(da)))
        return dq, dr, da

    def close(self):
        if self._h:
            lib().bsl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_precision(self, precision):
        _check(lib().bsl_set_precision(self._h, PREC[precision]))

    def set_kinetic_engine(self, engine):
        """Kinetic engine of the mixed precision: "simt" or "tensor"."""
        _check(lib().bsl_set_kinetic_engine(self._h, KINETIC[engine]))

    def set_kinetic_slices(self, slices):
        """9-bit slices kept by the tensor-core kinetic (1..4; 4 = exact)."""
        _check(lib().bsl_set_kinetic_slices(self._h, slices))

    def set_potential_format(self, fmt):
        """Potential blocks of the mixed path: "gaunt" (spherical-harmonic
        coefficients, the default where the basis has them), "fp32" or "bf16"
        (per-point scale)."""
        _check(lib().bsl_set_potential_format(self._h, VFORMAT[fmt]))

    def potential_format(self):
        f = lib().bsl_potential_format(self._h)
        if f < 0:
            raise BslError(ERR_STATE, "closed handle")
        return {v: k for k, v in VFORMAT.items()}[f]

    def gaunt_residual(self):
        """Largest |FP64 block element - its spherical-harmonic expansion| (kJ/mol), -1 if none."""
        return lib().bsl_gaunt_residual(self._h)

    def kinetic_engine(self):
        e = lib().bsl_kinetic_engine(self._h)
        if e < 0:
            raise BslError(ERR_STATE, "closed handle")
        return {v: k for k, v in KINETIC.items()}[e]

    def hv(self, vec, uec):
        """uec += H vec (host arrays, reference layout)."""
        _check(lib().bsl_hv_apply(self._h, _ptr(vec), _ptr(uec)))

    def hv_device(self, d_v, d_u, stream=0):
        """u = H v on device pointers in the packed layout."""
        _check(lib().bsl_hv_apply_device(self._h, C.c_void_p(d_v), C.c_void_p(d_u), C.c_void_p(stream)))

    def stream(self):
        return lib().bsl_stream(self._h)

    def inject_timeout(self, kernel_mask):
        """Test hook (bsl_debug_inject_timeout): later runs start with the
        time-out of the potential stream (bit 0) or of the tensor-core kinetic
        (bit 1) already recorded; 0 clears it."""
        _check(lib().bsl_debug_inject_timeout(self._h, kernel_mask))

    def lanczos(self, niter, start="uniform", seed=0):
        a = np.zeros(niter)
        b = np.zeros(niter + 1)
        b2 = np.zeros(niter + 1)
        _check(lib().bsl_lanczos_run(self._h, niter, START[start], seed, _ptr(a), _ptr(b), _ptr(b2)))
        return a, b, b2

    def last_ms_per_iter(self):
        x = np.zeros(1)
        _check(lib().bsl_last_run_ms_per_iter(self._h, _ptr(x)))
        return float(x[0])

    def step_host(self, vec, rvec):
        """One reference loop-body iteration on host state; returns alpha, beta, beta2."""
        out = np.zeros(3)
        o = out.ctypes.data
        _check(lib().bsl_lanczos_step_host(self._h, _ptr(vec), _ptr(rvec), C.cast(o, _P), C.cast(o + 8, _P),
                                           C.cast(o + 16, _P)))
        return out[0], out[1], out[2]

    def ritz(self, niter, evtr_rows, start=None, seed=0):
        """Ritz vectors (reference layout), evtr_rows[n] = T_m eigenvector n; `start`
        (and seed) as in the loop-1 run (default: the reference's uniform start)."""
        ng = evtr_rows.shape[0]
        ev = np.ascontiguousarray(evtr_rows, dtype=np.float64).reshape(-1)
        out = np.zeros(ng * self.basis_size)
        if start is None:
            _check(lib().bsl_ritz_vectors(self._h, niter, _ptr(ev), ng, _ptr(out)))
        else:
            _check(lib().bsl_ritz_vectors_start(self._h, niter, START[start], seed, _ptr(ev), ng, _ptr(out)))
        return out.reshape(ng, self.basis_size)

    def vgrid(self):
        n = lib().bsl_vgrid_size(self._h)
        a, b = np.zeros(n), np.zeros(n)
        _check(lib().bsl_copy_vgrid(self._h, _ptr(a), _ptr(b)))
        return a, b

    def vblocks(self):
        out = np.zeros(lib().bsl_vblock_size(self._h))
        _check(lib().bsl_copy_vblocks(self._h, _ptr(out)))
        return out


class _Storage:
    def __init__(self, calculator):
        self.calculator = calculator
        self.h = None
        self.total_basis_size = None


def hv_interface_setup(calculator):
    """Mirror of HvInterfaceSetup (interface.cpp:3): returns (storage, HvPrep, Hv).

    HvPrep(argv, storage) reads argv[2] (HvInputFile) and argv[3] (oscillator
    file) like the reference; Hv(argv, storage, vec, uec) accumulates
    uec += H vec.  Unknown names raise, where the reference prints and exits.
    """
    if calculator not in CALCULATORS:
        raise BslError(ERR_INPUT, "HvCalculator '%s' not recognized." % calculator)
    st = _Storage(calculator)

    def hv_prep(argv, storage, precision=os.environ.get("BSL_PRECISION", "fp64")):
        extra = argv[3] if len(argv) > 3 else None
        storage.h = Hamiltonian(argv[2], calculator, extra_input=extra, precision=precision)
        storage.total_basis_size = storage.h.basis_size
        return storage.total_basis_size

    def hv(argv, storage, vec, uec):
        storage.h.hv(vec, uec)

    return st, hv_prep, hv


def read_cage_xyz(path):
    """Molecules of a reference cage file: (centres of mass [nmol, 3] in Angstrom,
    ZYZ Euler angles [nmol, 3]) (the reader of SPCE_AH2_EngRoutines.cpp:5-108)."""
    with open(path) as f:
        lines = f.read().split("\n")
    nmol = int(lines[0].split()[0])
    cm, ea = np.zeros((nmol, 3)), np.zeros((nmol, 3))
    toks = " ".join(lines[2:]).split()
    for m in range(nmol):
        v = [float(x) for x in toks[7 * m + 1:7 * m + 7]]
        cm[m] = v[0::2]
        ea[m] = v[1::2]
    return cm, ea


def cage_levels_function():
    """torch.autograd.Function: the lowest levels of H2 in an SPC/E cage as a
    differentiable function of the cage (centres of mass [nmol, 3] in Angstrom,
    Euler angles [nmol, 3], site charges [3 nmol], Alavi H2 charges [2]).
    forward runs HvPrep, Lanczos loop 1, the eigen-tail, loop 2 (Ritz vectors)
    and the Hellmann-Feynman derivatives on the GPU; backward contracts them."""
    import torch

    class CageLevels(torch.autograd.Function):
        @staticmethod
        def forward(ctx, cm, euler, q_site, q_alavi, setup):
            precision = setup.get("precision", "fp64")
            niter, nlev = setup["niter"], setup["nlev"]
            cm_np, ea_np = cm.detach().cpu().double().numpy(), euler.detach().cpu().double().numpy()
            pot = setup.get("potential", POT_ALAVI_SPCE)
            h = Hamiltonian.from_cage(setup["params"], cm_np, ea_np, q_site.detach().cpu().double().numpy(),
                                      q_alavi.detach().cpu().double().numpy(), precision=precision,
                                      device=setup.get("device", 0), potential=pot)
            try:
                a, b, b2 = h.lanczos(niter, start="normal", seed=setup.get("seed", 0))
                mixed = precision == "mixed"
                ev, _ = good_eigenvalues(a, b, b2, setup.get("emin", -1e3), setup.get("emax", 1e3),
                                         MIXED_UNIT_ROUNDOFF if mixed else None, MIXED_REL_NOISE if mixed else None)
                if len(ev) < nlev:
                    raise BslError(ERR_INPUT, "only %d good eigenvalues, %d requested" % (len(ev), nlev))
                ev = ev[:nlev]
                rows = tm_eigenvectors(a, b, b2, ev)
                psi = h.ritz(niter, rows, start="normal", seed=setup.get("seed", 0))
                dq, dr, da = h.hf_gradient(psi, sites_per_molecule(pot) * cm_np.shape[0])
            finally:
                h.close()
            dcm, dea = rigid_body_gradient(cm_np, ea_np, dr, setup.get("potential", POT_ALAVI_SPCE))
            ctx.save_for_backward(torch.from_numpy(dcm), torch.from_numpy(dea), torch.from_numpy(dq),
                                  torch.from_numpy(da))
            return torch.from_numpy(np.ascontiguousarray(ev))

        @staticmethod
        def backward(ctx, gE):
            dcm, dea, dq, da = ctx.saved_tensors
            g = gE.to(torch.float64)
            return (torch.einsum("n,nmk->mk", g, dcm), torch.einsum("n,nmk->mk", g, dea),
                    torch.einsum("n,nw->w", g, dq), torch.einsum("n,na->a", g, da), None)

    return CageLevels
