"""Reference-format input files and the synthetic dodecahedral SPC/E cages.

The reference reads three whitespace-token files whose value order matters and
whose key names are ignored:
  * LanczosInputFile: 2 comment lines + 7 key/value pairs
    (headLoop/LanczosCode/lanczosEigenValuesVectors.cpp:33-69)
  * HvInputFile: 2 comment lines + 22 key/value pairs
    (Hv-calculators/linRotor/cartSphBasis/HvCalc/NoQuadOnTheFly/linRotCartSphHvFullVPrepRoutines.cpp:246-320)
  * cage .xyz: count, comment, then `name CMx phi CMy theta CMz chi` with the
    centre of mass in Angstrom and ZY'Z'' Euler angles in radians
    (Hv-calculators/linRotor/cartSphBasis/potentialCalc/Alavi/SPCE/SPCE_AH2_EngRoutines.cpp:17-38)

The synthetic cages place the 20 SPC/E oxygens on the vertices of a regular
dodecahedron (circumradius 3.95 Angstrom unless given), draw the Euler angles
uniformly (phi, chi in [0, 2pi), theta in [0, pi]) from numpy's PCG64 with the
given seed, and put each molecule's centre of mass at O_vertex - R * O_body so
that the oxygen sits exactly on the vertex.
"""
import math
import numpy as np

# SPC/E body-frame oxygen (nm), SPCE_AH2_EngRoutines.h:20-22
_O_BODY_NM = np.array([0.0, 0.0, 0.006461408220])


def rot_zyz(phi, theta, chi):
    """ZY'Z'' rotation matrix with the element formulas of rotmat.cpp:6-32."""
    cp, sp = math.cos(phi), math.sin(phi)
    ct, st = math.cos(theta), math.sin(theta)
    cx, sx = math.cos(chi), math.sin(chi)
    return np.array([[cp * ct * cx - sp * sx, -cp * ct * sx - sp * cx, cp * st],
                     [sp * ct * cx + cp * sx, -sp * ct * sx + cp * cx, sp * st],
                     [-st * cx, st * sx, ct]])


def dodecahedron_vertices(radius):
    g = (1.0 + math.sqrt(5.0)) / 2.0
    v = []
    for sx in (-1, 1):
        for sy in (-1, 1):
            for sz in (-1, 1):
                v.append((sx, sy, sz))
    for s1 in (-1, 1):
        for s2 in (-1, 1):
            v.append((0.0, s1 / g, s2 * g))
            v.append((s1 / g, s2 * g, 0.0))
            v.append((s1 * g, 0.0, s2 / g))
    v = np.array(v, dtype=np.float64)
    return v * (radius / math.sqrt(3.0))


def dodecahedral_cage(seed, radius=3.95):
    """20 waters: list of (name, cm_angstrom[3], euler[3])."""
    rng = np.random.default_rng(seed)
    out = []
    for i, o in enumerate(dodecahedron_vertices(radius)):
        phi = rng.uniform(0.0, 2.0 * math.pi)
        theta = rng.uniform(0.0, math.pi)
        chi = rng.uniform(0.0, 2.0 * math.pi)
        r = rot_zyz(phi, theta, chi)
        cm = o - (r @ _O_BODY_NM) * 10.0  # nm -> Angstrom
        out.append(("H2O%d" % (i + 1), cm, (phi, theta, chi)))
    return out


def write_cage_xyz(path, waters):
    with open(path, "w") as f:
        f.write("%d\n" % len(waters))
        f.write("# Format: [name_id]; CM-x (A); phi (rad); CM-y (A); theta (rad); CM-z (A); chi (rad); "
                "Euler angles for ZY'Z'' convention\n")
        for name, cm, ea in waters:
            f.write("%s %.17g %.17g %.17g %.17g %.17g %.17g\n" % (name, cm[0], ea[0], cm[1], ea[1], cm[2], ea[2]))


HV_KEYS = ["nx", "x_max(nm)", "ny", "y_max(nm)", "nz", "z_max(nm)", "l_max", "thetaPoints", "phiPoints",
           "pointPotential_nx", "pointPotential_x_max(nm)", "pointPotential_ny", "pointPotential_y_max(nm)",
           "pointPotential_nz", "pointPotential_z_max(nm)", "totalMass(g/mol)", "rotationalConstant(kJ/mol)",
           "geometryFilename", "simulationTitle", "ceilingPotential(kJ/mol)",
           "quadratureConvergenceStudy(TRUE/FALSE)", "rotationalSymmetry(All/Even/Odd)"]


def hv_fields(n, x_max, l_max, theta_points, phi_points, geometry, title, sym,
              total_mass=2.01588, rot_const=0.709648713, ceiling=18.0, point_grid=None):
    """Field values in HvInputFile order for a cubic grid.  point_grid = (points,
    width) of the potential universe the point-grid calculators tabulate the H2
    site energies on (default: the basis grid itself)."""
    pn, pmax = point_grid if point_grid else (n, x_max)
    return [n, x_max, n, x_max, n, x_max, l_max, theta_points, phi_points, pn, pmax, pn, pmax, pn, pmax,
            total_mass, rot_const, geometry, title, ceiling, "FALSE", sym]


def write_hv_input(path, values):
    with open(path, "w") as f:
        f.write("#\n#HvInputFile (reference token format; key names are ignored, order matters)\n")
        for k, v in zip(HV_KEYS, values):
            f.write("%s= %s\n" % (k, repr(v) if isinstance(v, float) else v))


def write_lanczos_input(path, niter, calculator, out_dir="./", emin=-10.0, emax=10.0, eigvec_word="none",
                        n_eigvec=0):
    keys = ["numberOfIterations", "EigenvalueOpenLowerLimit(kJ/mol)", "EigenvalueClosedUpperLimit(kJ/mol)",
            "NumberOfEigenvectors(all/partial/none)", "NumberOfEigenvectors", "HvCalculator",
            "OutputDirectoryPath"]
    vals = [niter, emin, emax, eigvec_word, n_eigvec, calculator, out_dir]
    with open(path, "w") as f:
        f.write("#LanczosInputFile (reference token format)\n#\n")
        for k, v in zip(keys, vals):
            f.write("%s= %s\n" % (k, v))


def write_isoharmosc_input(path, mass, frequency, max_energy):
    """Potential file read as argv[3] (IsoHarmOsc_Routines.cpp:41-58)."""
    with open(path, "w") as f:
        f.write("#\n#IsoHarmOsc input\n")
        f.write("mass(g/mol)= %r\nfrequency(1/ps)= %r\nmaxEnergy(kJ/mol)= %r\n" % (mass, frequency, max_energy))


def write_coulomb_input(path, centre_charge, mol_charge, ceiling):
    """Potential file read as argv[3] by the Coulomb calculator
    (Coulomb_Routines.cpp:36-85): two comment lines, then the charge at the
    origin, the charge on the H2 centre of mass (e) and the |V| ceiling (kJ/mol)."""
    with open(path, "w") as f:
        f.write("#\n#Coulomb input\n")
        f.write("centreCharge(e)= %r\nmolCharge(e)= %r\ncoulombPotentialCeiling(kJ/mol)= %r\n"
                % (centre_charge, mol_charge, ceiling))


# The two workloads: a CPU-sized parity case and the full-size metric case.
# x_max is the full box width (grid spans [-x_max/2, x_max/2]).
CONFIG_CPU = dict(name="15^3 even l<=4 12x24 (para)", n=15, x_max=0.08, l_max=4, theta_points=12, phi_points=12,
                  sym="Even", cage_seed=0, niter=600, levels=20)
CONFIG_METRIC = dict(name="54^3 odd l<=5 40x70 (ortho)", n=54, x_max=0.08, l_max=5, theta_points=40,
                     phi_points=35, sym="Odd", cage_seed=1, niter=10000, levels=40)


# The batched workload: 16 cages x {ortho, para} = 32 independent problems of
# uneven size, 24 theta x 48 phi, 3000 iterations each.
BATCH_EDGES = (27, 33, 41)


def batch_problems(ncages=16, edge_seed=3):
    """The 32 problems of the batched workload, as dicts: cage seeds 0..ncages-1,
    each cage's circumradius drawn uniformly from [3.85, 4.05] A (generator
    seeded with (cage seed, 1); the water orientations come from the cage seed
    as in dodecahedral_cage), each cage in the ortho (odd l <= 5, 21
    functions) and the para (even l <= 4, 15 functions) block, the grid edge of
    every run drawn from BATCH_EDGES (generator seeded with edge_seed)."""
    edges = np.random.default_rng(edge_seed).choice(BATCH_EDGES, size=2 * ncages)
    out = []
    for c in range(ncages):
        radius = float(np.random.default_rng([c, 1]).uniform(3.85, 4.05))
        for k, (sym, lmax) in enumerate((("Odd", 5), ("Even", 4))):
            out.append(dict(cage_seed=c, radius=radius, sym=sym, l_max=lmax, n=int(edges[2 * c + k]),
                            x_max=0.08, theta_points=24, phi_points=24, niter=3000))
    return out
