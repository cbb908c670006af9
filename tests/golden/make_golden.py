"""Generate the golden fixtures in tests/golden/ by running the EMerge reference.

Run with the path of an EMerge checkout (the directory that holds ``fem/``):

    python tests/golden/make_golden.py --ref /root/reference [fixture ...]

(or set EMERGE_REF_ROOT instead of passing ``--ref``).

The reference runs unmodified behind the import shims of ``_refshim`` (Numba
kernels execute as plain Python, gmsh is replaced by a fake that serves the
project's structured meshes).  Every fixture records the exact inputs the
reference saw, so the tests can replay them through the oracle and through the
CUDA path without the reference being present.

Fixtures:
  tet_elements.npz   ned2_tet_stiff_mass on 48 tets (fem/mth/tet.py:854-1088)
  tri_elements.npz   ned2_tri_stiff_force / ned2_tri_stiff (fem/mth/tri.py:575-797)
  small_assembly.npz tet_mass_stiffness_matrices on a 2x2x2-hex box, two material sets
                     (fem/physics/edm/optimized_assembly.py:43-116)
  waveguide.npz      WR-90 straight guide, h = 3 mm, 10 GHz: K row checksums, port
                     vectors, solve_ids, SuperLU field and S-parameters
                     (fem/physics/edm/assembler.py:312-388, fem/solver.py:405-469,
                     fem/physics/edm/emfreq3d.py:607-779)
  waveguide_abc.npz  the same guide with port 2 replaced by an AbsorbingBoundary:
                     K row checksums, solve_ids, port vector at 10 GHz
  interp.npz         ned2_tet_interp (fem/mth/tet.py:372-497) of the guide's 10 GHz
                     SuperLU field: 6-point quadrature points of the port-1 triangles
                     over the port tets (the S-parameter evaluation) and random
                     interior points over all tets
  lumped.npz         parallel-plate line between two LumpedPorts (fem/bc.py:620-745) with
                     absorbing side walls, 10 GHz: K and port-vector checksums, the
                     voltage lines of define_lumped_port_integration_points
                     (fem/physics/edm/emfreq3d.py:366-389), SuperLU fields and the
                     voltage-integral S-parameters (emfreq3d.py:752-766)
  frames.npz         Axis.construct_cs (fem/cs.py:63-70): the port frames of 18 face normals
  port_elements.npz  generalized_matrix_GQ (fem/physics/edm/nedeleclegrange2.py:224-382), the
                     14x14 element matrices of the 2-D port mode problem, on 24 triangles with
                     random edge orientations and isotropic / anisotropic materials
  waveguide_k.npz    K(k0) of the waveguide at 10 GHz entry by entry on the port-face rows
                     and 1500 random rows (fem/physics/edm/assembler.py:312-388)
  waveguide_diel.npz the guide with a lossy dielectric at port 1: SuperLU fields and the
                     S-parameters with the per-triangle material weight of the mode
                     integrals (fem/physics/edm/emfreq3d.py:767-778)
  port_interp.npz    ned2_tri_interp_full / ned2_tri_interp_curl (fem/mth/tri.py:228-401) of
                     random port fields on the WR-90 port face, at quadrature and random points
  farfield.npz       stratton_chu (fem/physics/edm/sc.py:143-180) of a short dipole's
                     near field sampled at the edge centres of a closed box surface
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _refshim  # noqa: E402

# ``--ref PATH``: the EMerge checkout to run (else EMERGE_REF_ROOT)
_ARGS = sys.argv[1:]
if "--ref" in _ARGS:
    _i = _ARGS.index("--ref")
    _refshim.REF_ROOT = _ARGS[_i + 1]
    del _ARGS[_i:_i + 2]
GMSH = _refshim.install()

from fem.mth import tet as ref_tet  # noqa: E402
from fem.mth import tri as ref_tri  # noqa: E402
from fem.mth import optimized as ref_opt  # noqa: E402
from fem import mesh3d as ref_mesh3d  # noqa: E402
from fem.elements.nedelec2 import Nedelec2  # noqa: E402
from fem.physics.edm import optimized_assembly as ref_asm  # noqa: E402
from fem.physics.edm import assembler as ref_assembler  # noqa: E402
from fem.physics.edm.emfreq3d import Electrodynamics3D  # noqa: E402
from fem import solver as ref_solver  # noqa: E402
from fem import bc as ref_bc  # noqa: E402
from fem.cs import CoordinateSystem, Axis  # noqa: E402
from fem.selection import FaceSelection  # noqa: E402

from emerge_gb300.mesh import structured_box, TET_EDGE_SLOTS, TET_FACE_SLOTS  # noqa: E402
from emerge_gb300 import mesh as pm  # noqa: E402

C0 = 299792458


def _local_maps(gid):
    """local_edge_map / local_tri_map of a tet whose vertices have global ids ``gid``."""
    ge = np.array([[min(gid[p], gid[q]), max(gid[p], gid[q])] for p, q in TET_EDGE_SLOTS.T]).T
    gf = np.array([sorted([gid[a], gid[b], gid[c]]) for a, b, c in TET_FACE_SLOTS.T]).T
    lem = ref_opt.local_mapping(np.asarray(gid, dtype=np.int64), ge.astype(np.int64))
    ltm = ref_opt.local_mapping(np.asarray(gid, dtype=np.int64), gf.astype(np.int64))
    return lem, ltm


def _rand_c3(rng, iso):
    if iso:
        return (rng.uniform(0.5, 10) - 1j * rng.uniform(0, 0.2)) * np.eye(3, dtype=np.complex128)
    return (rng.normal(size=(3, 3)) + 1j * rng.normal(size=(3, 3)) * 0.3 + 3 * np.eye(3)).astype(np.complex128)


def make_tet_elements():
    rng = np.random.default_rng(1234)
    n = 48
    verts = np.zeros((n, 3, 4))
    lens = np.zeros((n, 6))
    lem = np.zeros((n, 2, 6), dtype=np.int64)
    ltm = np.zeros((n, 3, 4), dtype=np.int64)
    Ms = np.zeros((n, 3, 3), dtype=np.complex128)
    Mm = np.zeros((n, 3, 3), dtype=np.complex128)
    D = np.zeros((n, 20, 20), dtype=np.complex128)
    F = np.zeros((n, 20, 20), dtype=np.complex128)
    for k in range(n):
        scale = [1.0, 1e-3, 3e-3, 0.0125][k % 4]
        offset = [0.0, 0.0, 0.02, 0.9][k % 4]
        v = offset + scale * (np.array([[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=float)
                              + 0.3 * rng.uniform(-1, 1, size=(3, 4)))
        gid = rng.choice(1000, size=4, replace=False)
        lem[k], ltm[k] = _local_maps(gid)
        verts[k] = v
        for s, (p, q) in enumerate(TET_EDGE_SLOTS.T):
            lens[k, s] = np.sqrt(np.sum((v[:, p] - v[:, q]) ** 2))
        Ms[k] = _rand_c3(rng, k % 3 != 2)
        Mm[k] = _rand_c3(rng, k % 3 != 1)
        D[k], F[k] = ref_tet.ned2_tet_stiff_mass(verts[k], lens[k], lem[k], ltm[k], Ms[k], Mm[k])
    np.savez_compressed(os.path.join(HERE, "tet_elements.npz"), verts=verts, edge_lengths=lens,
                        local_edge_map=lem, local_tri_map=ltm, Ms=Ms, Mm=Mm, D=D, F=F)
    print("tet_elements: ok")


def make_tri_elements():
    rng = np.random.default_rng(99)
    n = 24
    DPTs = ref_opt.gaus_quad_tri(4)
    lv = np.zeros((n, 3, 3))
    gam = np.zeros(n, dtype=np.complex128)
    U = np.zeros((n, 3, DPTs.shape[1]), dtype=np.complex128)
    Bf = np.zeros((n, 8, 8), dtype=np.complex128)
    bf = np.zeros((n, 8), dtype=np.complex128)
    v3 = np.zeros((n, 3, 3))
    el = np.zeros((n, 3))
    Bs = np.zeros((n, 8, 8), dtype=np.complex128)
    for k in range(n):
        s = [1e-3, 2e-3, 1.0][k % 3]
        lv[k] = s * (np.array([[0, 1, 0], [0, 0, 1], [0, 0, 0]], dtype=float) + 0.3 * rng.uniform(-1, 1, (3, 3)))
        lv[k, 2] = rng.uniform(-1, 1, 3) * s * 0.01
        gam[k] = 1j * rng.uniform(50, 300) + rng.uniform(-1, 1)
        U[k] = rng.normal(size=(3, DPTs.shape[1])) + 1j * rng.normal(size=(3, DPTs.shape[1]))
        Bf[k], bf[k] = ref_tri.ned2_tri_stiff_force(lv[k], gam[k], U[k], DPTs)
        v3[k] = s * (np.eye(3) + 0.3 * rng.uniform(-1, 1, (3, 3))) + rng.uniform(-1, 1, (3, 1)) * s
        el[k] = [np.linalg.norm(v3[k][:, a] - v3[k][:, b]) for a, b in ((0, 1), (1, 2), (0, 2))]
        Bs[k] = ref_tri.ned2_tri_stiff(v3[k], el[k], gam[k])
    np.savez_compressed(os.path.join(HERE, "tri_elements.npz"), lcs_vertices=lv, gamma=gam, Uinc=U,
                        DPTs=DPTs, B_force=Bf, b_force=bf, vertices=v3, edge_lengths=el, B_stiff=Bs)
    print("tri_elements: ok")


def reference_mesh(tm):
    """Run the reference Mesh3D.update on a project mesh through the fake gmsh."""
    GMSH.set_mesh(tm.nodes, tm.tets, tm.boundary, tm.cell_tag)
    m = ref_mesh3d.Mesh3D(None)
    m.update()
    return m


def mesh_arrays(m, prefix=""):
    return {prefix + "nodes": m.nodes, prefix + "tets": m.tets.astype(np.int32),
            prefix + "edges": m.edges.astype(np.int32), prefix + "tris": m.tris.astype(np.int32),
            prefix + "tet_to_edge": m.tet_to_edge.astype(np.int32),
            prefix + "tet_to_tri": m.tet_to_tri.astype(np.int32),
            prefix + "tri_to_edge": m.tri_to_edge.astype(np.int32),
            prefix + "tri_to_tet": m.tri_to_tet.astype(np.int32),
            prefix + "edge_lengths": m.edge_lengths}


def make_small_assembly():
    rng = np.random.default_rng(7)
    xs = np.array([0.0, 0.4, 1.0])
    tm = structured_box(xs, xs * 0.8, xs * 1.3 + 0.5, jitter=0.15, seed=3)
    m = reference_mesh(tm)
    field = Nedelec2(m)
    nT = m.n_tets
    out = mesh_arrays(m)
    out["tet_to_field"] = field.tet_to_field.astype(np.int32)
    for tag, iso_mu in (("a", True), ("b", False)):
        er = np.zeros((3, 3, nT), dtype=np.complex128)
        ur = np.zeros((3, 3, nT), dtype=np.complex128)
        for t in range(nT):
            er[:, :, t] = rng.uniform(1, 10) * (1 - 1j * rng.uniform(0.001, 0.02)) * np.eye(3)
            ur[:, :, t] = np.eye(3) if iso_mu else rng.uniform(0.5, 3) * np.eye(3)
        t0 = time.time()
        E, B = ref_asm.tet_mass_stiffness_matrices(field, er, ur)
        print(f"small_assembly[{tag}]: {nT} tets in {time.time() - t0:.1f} s, N={E.shape[0]}, nnz={E.nnz}")
        out[f"er_{tag}"] = er
        out[f"ur_{tag}"] = ur
        for name, M in (("E", E), ("B", B)):
            out[f"{name}_{tag}_indptr"] = M.indptr.astype(np.int64)
            out[f"{name}_{tag}_indices"] = M.indices.astype(np.int32)
            out[f"{name}_{tag}_data"] = M.data
    np.savez_compressed(os.path.join(HERE, "small_assembly.npz"), **out)


def waveguide_mesh(h=3e-3):
    a, b, L = 0.02286, 0.01016, 0.05
    nx, ny, nz = int(np.ceil(a / h)), int(np.ceil(L / h)), int(np.ceil(b / h))
    return structured_box(np.linspace(0, a, nx + 1), np.linspace(0, L, ny + 1), np.linspace(0, b, nz + 1)), (a, b, L)


def make_waveguide():
    tm, (a, b, L) = waveguide_mesh()
    m = reference_mesh(tm)
    field = Nedelec2(m)
    nT = m.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    ur = er.copy()
    p1 = ref_bc.RectangularWaveguide(FaceSelection([pm.FACE_YMIN]), 1, cs=CoordinateSystem(
        Axis(np.array([1.0, 0, 0])), Axis(np.array([0, 0, 1.0])), Axis(np.array([0, -1.0, 0])),
        np.array([a / 2, 0.0, b / 2])), dims=(a, b))
    p2 = ref_bc.RectangularWaveguide(FaceSelection([pm.FACE_YMAX]), 2, cs=CoordinateSystem(
        Axis(np.array([-1.0, 0, 0])), Axis(np.array([0, 0, 1.0])), Axis(np.array([0, 1.0, 0])),
        np.array([a / 2, L, b / 2])), dims=(a, b))
    # the reference stores ``dims`` only when it derives them itself (fem/bc.py:538-546)
    p1.dims = (a, b)
    p2.dims = (a, b)
    pec = ref_bc.PEC(FaceSelection([pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX]))
    bcs = [pec, p1, p2]
    asm = ref_assembler.Assembler()
    freqs = [9.0e9, 10.0e9]
    routine = ref_solver.SolveRoutine(ref_solver.ReverseCuthillMckee(), ref_solver.Preconditioner(), None,
                                      ref_solver.SolverSuperLU(), None, None)
    routine.use_preconditioner = False
    phys = Electrodynamics3D.__new__(Electrodynamics3D)
    phys.mesh = m
    all_ports = [p1, p2]
    verts = set()
    for p in all_ports:
        tris = m.get_triangles(p.tags)
        p._tri_ids = tris
        p._tri_vertices = m.tris[:, tris]
        verts.update(set(p._tri_vertices.ravel().tolist()))
    port_tets = np.array([t for t in range(nT) if not set(m.tets[:, t].tolist()).isdisjoint(verts)])
    out = mesh_arrays(m)
    out["tet_to_field"] = field.tet_to_field.astype(np.int32)
    out["tri_to_field"] = field.tri_to_field.astype(np.int32)
    out["freqs"] = np.array(freqs)
    out["dims"] = np.array([a, b, L])
    out["port_tris_1"] = p1._tri_ids.astype(np.int32)
    out["port_tris_2"] = p2._tri_ids.astype(np.int32)
    out["pec_tris"] = m.get_triangles(pec.tags).astype(np.int32)
    S = np.zeros((len(freqs), 2, 2), dtype=np.complex128)
    t0 = time.time()
    for fi, f in enumerate(freqs):
        k0 = 2 * np.pi * f / C0
        K, bvec, solve_ids, pvecs = asm.assemble_freq_matrix(field, er, ur, bcs, f, cache_matrices=True)
        if fi == 0:
            E, B = asm.cached_matrices
            n = E.shape[0]
            w = (np.arange(n) + 1.0) / n
            for name, M in (("E", E), ("B", B)):
                out[f"{name}_nnz"] = np.int64(M.nnz)
                out[f"{name}_rowsum"] = np.asarray(M.sum(axis=1)).ravel()
                out[f"{name}_rowmom"] = M @ w
                out[f"{name}_indptr"] = M.indptr.astype(np.int64)
            out["solve_ids"] = solve_ids.astype(np.int32)
        Kc = K.tocsr()
        out[f"K{fi}_rowsum"] = np.asarray(Kc.sum(axis=1)).ravel()
        out[f"K{fi}_rowmom"] = Kc @ ((np.arange(Kc.shape[0]) + 1.0) / Kc.shape[0])
        for pn in (1, 2):
            nz = np.nonzero(pvecs[pn])[0]
            out[f"pvec{fi}_{pn}_idx"] = nz.astype(np.int32)
            out[f"pvec{fi}_{pn}_val"] = pvecs[pn][nz]
        for active in all_ports:
            active.active = True
            sol = routine.solve(K, bvec + pvecs[active.port_number], solve_ids, reuse=False)
            out[f"x{fi}_{active.port_number}"] = sol
            fieldf = field.interpolate_Ef(sol, tetids=port_tets)
            ones = np.ones((3, 3, 0))
            pf, pmode = phys._compute_s_data(active, fieldf, active._tri_vertices, k0,
                                             np.repeat(np.eye(3)[:, :, None], len(active._tri_ids), 2),
                                             np.repeat(np.eye(3)[:, :, None], len(active._tri_ids), 2))
            for bcp in all_ports:
                pf, _ = phys._compute_s_data(bcp, fieldf, bcp._tri_vertices, k0,
                                             np.repeat(np.eye(3)[:, :, None], len(bcp._tri_ids), 2),
                                             np.repeat(np.eye(3)[:, :, None], len(bcp._tri_ids), 2))
                S[fi, bcp.port_number - 1, active.port_number - 1] = pf / pmode
            active.active = False
        print(f"waveguide f={f / 1e9:.1f} GHz: |S11|={abs(S[fi, 0, 0]):.4f} |S21|={abs(S[fi, 1, 0]):.4f} "
              f"({time.time() - t0:.1f} s)")
    out["S"] = S
    out["port_tets"] = port_tets.astype(np.int32)
    np.savez_compressed(os.path.join(HERE, "waveguide.npz"), **out)


def _guide_ports(m, a, b, L):
    p1 = ref_bc.RectangularWaveguide(FaceSelection([pm.FACE_YMIN]), 1, cs=CoordinateSystem(
        Axis(np.array([1.0, 0, 0])), Axis(np.array([0, 0, 1.0])), Axis(np.array([0, -1.0, 0])),
        np.array([a / 2, 0.0, b / 2])), dims=(a, b))
    p2 = ref_bc.RectangularWaveguide(FaceSelection([pm.FACE_YMAX]), 2, cs=CoordinateSystem(
        Axis(np.array([-1.0, 0, 0])), Axis(np.array([0, 0, 1.0])), Axis(np.array([0, 1.0, 0])),
        np.array([a / 2, L, b / 2])), dims=(a, b))
    p1.dims = (a, b)
    p2.dims = (a, b)
    for p in (p1, p2):
        p._tri_ids = m.get_triangles(p.tags)
        p._tri_vertices = m.tris[:, p._tri_ids]
    pec = ref_bc.PEC(FaceSelection([pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX]))
    return p1, p2, pec


def make_waveguide_k():
    """Entry-by-entry K(k0) of the WR-90 guide at 10 GHz (assembler.py:312-388) on a row
    subset: every row of a port-face DOF (where the Robin blocks land) plus 1500 random
    rows.  The mesh is the one of waveguide.npz (checked)."""
    tm, (a, b, L) = waveguide_mesh()
    m = reference_mesh(tm)
    ref = np.load(os.path.join(HERE, "waveguide.npz"))
    assert np.array_equal(ref["tets"], m.tets) and np.array_equal(ref["edges"], m.edges)
    assert np.array_equal(ref["tris"], m.tris)
    field = Nedelec2(m)
    nT = m.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    ur = er.copy()
    p1, p2, pec = _guide_ports(m, a, b, L)
    asm = ref_assembler.Assembler()
    f = 10.0e9
    K, bvec, solve_ids, pvecs = asm.assemble_freq_matrix(field, er, ur, [pec, p1, p2], f, cache_matrices=True)
    Kc = K.tocsr()
    Kc.sort_indices()
    rng = np.random.default_rng(11)
    port_rows = np.unique(field.tri_to_field[:, np.r_[p1._tri_ids, p2._tri_ids]])
    rows = np.unique(np.r_[port_rows, rng.choice(Kc.shape[0], 1500, replace=False)]).astype(np.int64)
    sub = Kc[rows]
    np.savez_compressed(os.path.join(HERE, "waveguide_k.npz"), freq=np.float64(f), rows=rows,
                        port_rows=port_rows.astype(np.int64), indptr=sub.indptr.astype(np.int64),
                        indices=sub.indices.astype(np.int32), data=sub.data, nnz_total=np.int64(Kc.nnz))
    print(f"waveguide_k: {len(rows)} rows, {sub.nnz} entries of {Kc.nnz}")


def make_waveguide_diel():
    """WR-90 guide with its first 20 mm filled by a lossy dielectric (er = 2.2 - 0.02j), so the
    two waveports see different fills: the S-parameters carry the reference's per-triangle
    material weight of the mode integrals (emfreq3d.py:767-778, sparam.py:102-139), with the
    port-face materials taken from each face's first tet (emfreq3d.py:480-486)."""
    tm, (a, b, L) = waveguide_mesh()
    m = reference_mesh(tm)
    field = Nedelec2(m)
    nT = m.n_tets
    cy = m.nodes[1][m.tets].mean(axis=0)
    eps = np.where(cy < 0.02, 2.2 - 0.02j, 1.0 + 0j)
    er = np.eye(3, dtype=np.complex128)[:, :, None] * eps[None, None, :]
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    p1, p2, pec = _guide_ports(m, a, b, L)
    all_ports = [p1, p2]
    ertri = er[:, :, m.tri_to_tet[0]]
    urtri = ur[:, :, m.tri_to_tet[0]]
    verts = set()
    for p in all_ports:
        verts.update(set(p._tri_vertices.ravel().tolist()))
    port_tets = np.array([t for t in range(nT) if not set(m.tets[:, t].tolist()).isdisjoint(verts)])
    asm = ref_assembler.Assembler()
    routine = ref_solver.SolveRoutine(ref_solver.ReverseCuthillMckee(), ref_solver.Preconditioner(), None,
                                      ref_solver.SolverSuperLU(), None, None)
    routine.use_preconditioner = False
    phys = Electrodynamics3D.__new__(Electrodynamics3D)
    phys.mesh = m
    f = 10.0e9
    k0 = 2 * np.pi * f / C0
    K, bvec, solve_ids, pvecs = asm.assemble_freq_matrix(field, er, ur, [pec, p1, p2], f, cache_matrices=True)
    out = mesh_arrays(m)
    out["tet_to_field"] = field.tet_to_field.astype(np.int32)
    out["tri_to_field"] = field.tri_to_field.astype(np.int32)
    out["dims"] = np.array([a, b, L])
    out["freq"] = np.float64(f)
    out["eps"] = eps
    out["port_tris_1"] = p1._tri_ids.astype(np.int32)
    out["port_tris_2"] = p2._tri_ids.astype(np.int32)
    out["pec_tris"] = m.get_triangles(pec.tags).astype(np.int32)
    S = np.zeros((2, 2), dtype=np.complex128)
    for active in all_ports:
        active.active = True
        sol = routine.solve(K, bvec + pvecs[active.port_number], solve_ids, reuse=False)
        out[f"x_{active.port_number}"] = sol
        fieldf = field.interpolate_Ef(sol, tetids=port_tets)
        tr = active._tri_ids
        _, pmode = phys._compute_s_data(active, fieldf, active._tri_vertices, k0, ertri[:, :, tr], urtri[:, :, tr])
        for bcp in all_ports:
            tr = bcp._tri_ids
            pf, _ = phys._compute_s_data(bcp, fieldf, bcp._tri_vertices, k0, ertri[:, :, tr], urtri[:, :, tr])
            S[bcp.port_number - 1, active.port_number - 1] = pf / pmode
        active.active = False
    out["S"] = S
    np.savez_compressed(os.path.join(HERE, "waveguide_diel.npz"), **out)
    print(f"waveguide_diel: |S11|={abs(S[0, 0]):.4f} |S21|={abs(S[1, 0]):.4f} |S12|={abs(S[0, 1]):.4f}")


def make_port_interp():
    """ned2_tri_interp_full / ned2_tri_interp_curl (fem/mth/tri.py:228-401) of random port
    fields on the WR-90 port face of waveguide.npz's mesh, at the 6-point quadrature points
    of every face triangle and at random points of the face (local port coordinates)."""
    from emerge_gb300.modes import port_surface
    from emerge_gb300.bc import CoordinateSystem as PCS
    z = np.load(os.path.join(HERE, "waveguide.npz"))
    tri_ids = z["port_tris_1"].astype(np.int64)
    mesh = type("M", (), {})()
    mesh.tris = z["tris"].astype(np.int64)
    S = port_surface(mesh, tri_ids)
    a, b, L = (float(v) for v in z["dims"])
    cs = PCS([1.0, 0, 0], [0, 0, 1.0], [0, -1.0, 0], [a / 2, 0.0, b / 2])
    nodes = z["nodes"][:, S.node_ids]
    xl, yl, _ = cs.in_local_cs(nodes[0], nodes[1], nodes[2])
    nodes2 = np.stack([xl, yl])
    rng = np.random.default_rng(21)
    field = rng.normal(size=S.n_field) + 1j * rng.normal(size=S.n_field)
    nT = S.tris.shape[1]
    diadic = np.zeros((3, 3, nT), dtype=np.complex128)
    for k in range(3):
        diadic[k, k] = rng.uniform(0.5, 2, nT) + 1j * rng.uniform(-0.1, 0.1, nT)
    D = ref_opt.gaus_quad_tri(4)
    v = [nodes2[:, S.tris[k]] for k in range(3)]
    qp = np.concatenate([v[0] * D[1, q] + v[1] * D[2, q] + v[2] * D[3, q] for q in range(D.shape[1])], axis=1)
    rp = np.stack([rng.uniform(xl.min(), xl.max(), 200), rng.uniform(yl.min(), yl.max(), 200)])
    coords = np.ascontiguousarray(np.concatenate([qp, rp], axis=1))
    tris = np.ascontiguousarray(S.tris.astype(np.int64))
    t2f = np.ascontiguousarray(S.tri_to_field.astype(np.int64))
    Ex, Ey, Ez = ref_tri.ned2_tri_interp_full(coords, field, tris, np.ascontiguousarray(nodes2), t2f)
    beta = 157.3
    Hx, Hy, Hz = ref_tri.ned2_tri_interp_curl(coords, field, tris, np.ascontiguousarray(nodes2), t2f, diadic, beta)
    np.savez_compressed(os.path.join(HERE, "port_interp.npz"), coords=coords, field=field, tris=S.tris.astype(np.int32),
                        nodes2=nodes2, tri_to_field=S.tri_to_field.astype(np.int32),
                        diadic_diag=np.stack([diadic[0, 0], diadic[1, 1], diadic[2, 2]]), beta=np.float64(beta),
                        E=np.stack([Ex, Ey, Ez]), H=np.stack([Hx, Hy, Hz]))
    print(f"port_interp: {coords.shape[1]} points over {nT} triangles")


def make_waveguide_abc():
    """WR-90 guide with port 2 replaced by a first-order absorbing boundary
    (fem/bc.py:254-300, assemble_robin_bc fem/physics/edm/assembler.py:125-144)."""
    tm, (a, b, L) = waveguide_mesh()
    m = reference_mesh(tm)
    field = Nedelec2(m)
    nT = m.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    ur = er.copy()
    p1 = ref_bc.RectangularWaveguide(FaceSelection([pm.FACE_YMIN]), 1, cs=CoordinateSystem(
        Axis(np.array([1.0, 0, 0])), Axis(np.array([0, 0, 1.0])), Axis(np.array([0, -1.0, 0])),
        np.array([a / 2, 0.0, b / 2])), dims=(a, b))
    p1.dims = (a, b)
    abc = ref_bc.AbsorbingBoundary(FaceSelection([pm.FACE_YMAX]))
    pec = ref_bc.PEC(FaceSelection([pm.FACE_XMIN, pm.FACE_XMAX, pm.FACE_ZMIN, pm.FACE_ZMAX]))
    asm = ref_assembler.Assembler()
    f = 10.0e9
    K, bvec, solve_ids, pvecs = asm.assemble_freq_matrix(field, er, ur, [pec, p1, abc], f, cache_matrices=True)
    Kc = K.tocsr()
    n = Kc.shape[0]
    out = mesh_arrays(m)
    out["tet_to_field"] = field.tet_to_field.astype(np.int32)
    out["tri_to_field"] = field.tri_to_field.astype(np.int32)
    out["dims"] = np.array([a, b, L])
    out["freq"] = np.float64(f)
    out["port_tris_1"] = p1._tri_ids.astype(np.int32) if p1._tri_ids is not None else m.get_triangles(p1.tags).astype(np.int32)
    out["abc_tris"] = m.get_triangles(abc.tags).astype(np.int32)
    out["pec_tris"] = m.get_triangles(pec.tags).astype(np.int32)
    out["K_rowsum"] = np.asarray(Kc.sum(axis=1)).ravel()
    out["K_rowmom"] = Kc @ ((np.arange(n) + 1.0) / n)
    out["solve_ids"] = solve_ids.astype(np.int32)
    nz = np.nonzero(pvecs[1])[0]
    out["pvec_1_idx"] = nz.astype(np.int32)
    out["pvec_1_val"] = pvecs[1][nz]
    np.savez_compressed(os.path.join(HERE, "waveguide_abc.npz"), **out)
    print("waveguide_abc: ok")


def make_interp():
    """Reference field interpolation of the waveguide fixture's 10 GHz port-1 solution."""
    z = np.load(os.path.join(HERE, "waveguide.npz"))
    tm, (a, b, L) = waveguide_mesh()
    m = reference_mesh(tm)
    field = Nedelec2(m)
    sol = z["x1_1"]
    rng = np.random.default_rng(21)
    # port-1 quadrature points (6-point Dunavant rule, as the S-parameter integral uses)
    D = ref_opt.gaus_quad_tri(4)
    tri = np.asarray(z["port_tris_1"], dtype=np.int64)
    tv = m.tris[:, tri]
    v1, v2, v3 = m.nodes[:, tv[0]], m.nodes[:, tv[1]], m.nodes[:, tv[2]]
    pts = []
    for k in range(D.shape[1]):
        pts.append(v1 * D[1, k] + v2 * D[2, k] + v3 * D[3, k])
    port_pts = np.concatenate(pts, axis=1)
    # interior points: a random barycentric point of 300 random tets
    tsel = rng.choice(m.n_tets, 300, replace=False)
    lam = rng.dirichlet(np.ones(4), size=300).T * 0.9 + 0.025
    lam /= lam.sum(axis=0)
    inner = np.einsum("vt,dvt->dt", lam, m.nodes[:, m.tets[:, tsel]])
    port_tets = np.asarray(z["port_tets"], dtype=np.int64)
    t0 = time.time()
    Ep = field.interpolate(sol, port_pts[0], port_pts[1], port_pts[2], tetids=port_tets)
    Ei = field.interpolate(sol, inner[0], inner[1], inner[2], tetids=np.arange(m.n_tets, dtype=np.int64))
    print(f"interp: {port_pts.shape[1]} port points, {inner.shape[1]} interior points ({time.time() - t0:.1f} s)")
    np.savez_compressed(os.path.join(HERE, "interp.npz"), port_points=port_pts, port_tets=port_tets,
                        port_E=np.stack(Ep), inner_points=inner, inner_E=np.stack(Ei), inner_tets=tsel)


def lumped_mesh(h=1e-3):
    L, W, H = 0.015, 0.006, 0.002
    nx, ny, nz = int(round(L / h)), int(round(W / h)), int(round(H / h))
    return structured_box(np.linspace(0, L, nx + 1), np.linspace(0, W, ny + 1), np.linspace(0, H, nz + 1)), (L, W, H)


def make_lumped():
    """Two lumped ports (x = 0 and x = L faces, E along +z) on a parallel-plate line:
    PEC plates at z = 0 and z = H, first-order absorbing walls at y = 0 and y = W."""
    tm, (L, W, H) = lumped_mesh()
    m = reference_mesh(tm)
    GMSH.face_normals = {pm.FACE_XMIN: (-1.0, 0, 0), pm.FACE_XMAX: (1.0, 0, 0)}
    field = Nedelec2(m)
    nT = m.n_tets
    er = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2) * (2.2 - 0.01j)
    ur = np.repeat(np.eye(3, dtype=np.complex128)[:, :, None], nT, axis=2)
    from fem.cs import ZAX
    p1 = ref_bc.LumpedPort(FaceSelection([pm.FACE_XMIN]), 1, width=W, height=H, direction=ZAX, Z0=50.0)
    p2 = ref_bc.LumpedPort(FaceSelection([pm.FACE_XMAX]), 2, width=W, height=H, direction=ZAX, Z0=50.0)
    abc = ref_bc.AbsorbingBoundary(FaceSelection([pm.FACE_YMIN, pm.FACE_YMAX]))
    pec = ref_bc.PEC(FaceSelection([pm.FACE_ZMIN, pm.FACE_ZMAX]))
    bcs = [pec, abc, p1, p2]
    phys = Electrodynamics3D.__new__(Electrodynamics3D)
    phys.mesh = m
    for p in (p1, p2):
        phys.define_lumped_port_integration_points(p)
    asm = ref_assembler.Assembler()
    routine = ref_solver.SolveRoutine(ref_solver.ReverseCuthillMckee(), ref_solver.Preconditioner(), None,
                                      ref_solver.SolverSuperLU(), None, None)
    routine.use_preconditioner = False
    f = 10e9
    k0 = 2 * np.pi * f / C0
    K, bvec, solve_ids, pvecs = asm.assemble_freq_matrix(field, er, ur, bcs, f, cache_matrices=True)
    out = mesh_arrays(m)
    out["tet_to_field"] = field.tet_to_field.astype(np.int32)
    out["tri_to_field"] = field.tri_to_field.astype(np.int32)
    out["dims"] = np.array([L, W, H])
    out["freq"] = f
    out["er"] = np.complex128(2.2 - 0.01j)
    Kc = K.tocsr()
    out["K_rowsum"] = np.asarray(Kc.sum(axis=1)).ravel()
    out["K_rowmom"] = Kc @ ((np.arange(Kc.shape[0]) + 1.0) / Kc.shape[0])
    out["solve_ids"] = solve_ids.astype(np.int32)
    verts = set()
    for p in (p1, p2):
        tris = m.get_triangles(p.tags)
        p._tri_ids = tris
        p._tri_vertices = m.tris[:, tris]
        verts.update(set(p._tri_vertices.ravel().tolist()))
        out[f"port_tris_{p.port_number}"] = tris.astype(np.int32)
        nz = np.nonzero(pvecs[p.port_number])[0]
        out[f"pvec_{p.port_number}_idx"] = nz.astype(np.int32)
        out[f"pvec_{p.port_number}_val"] = pvecs[p.port_number][nz]
        ln = p.vintline
        out[f"line_{p.port_number}_mid"] = np.array(ln.cmid)
        out[f"line_{p.port_number}_d"] = np.array([ln.dxs, ln.dys, ln.dzs])
        out[f"gamma_{p.port_number}"] = np.complex128(p.get_gamma(k0))
    out["pec_tris"] = m.get_triangles(pec.tags).astype(np.int32)
    out["abc_tris"] = m.get_triangles(abc.tags).astype(np.int32)
    port_tets = np.array([t for t in range(nT) if not set(m.tets[:, t].tolist()).isdisjoint(verts)])
    out["port_tets"] = port_tets.astype(np.int32)
    S = np.zeros((2, 2), dtype=np.complex128)
    eye = lambda p: np.repeat(np.eye(3)[:, :, None], len(p._tri_ids), 2)  # noqa: E731
    for active in (p1, p2):
        active.active = True
        sol = routine.solve(K, bvec + pvecs[active.port_number], solve_ids, reuse=False)
        out[f"x_{active.port_number}"] = sol
        fieldf = field.interpolate_Ef(sol, tetids=port_tets)
        _, pmode = phys._compute_s_data(active, fieldf, active._tri_vertices, k0, eye(active), eye(active))
        for bcp in (p1, p2):
            pf, _ = phys._compute_s_data(bcp, fieldf, bcp._tri_vertices, k0, eye(bcp), eye(bcp))
            S[bcp.port_number - 1, active.port_number - 1] = pf / pmode
        active.active = False
    out["S"] = S
    print(f"lumped: {nT} tets, |S11|={abs(S[0, 0]):.4f} |S21|={abs(S[1, 0]):.4f}")
    np.savez_compressed(os.path.join(HERE, "lumped.npz"), **out)


def make_frames():
    """Port frames the reference builds from a face normal (Axis.construct_cs, fem/cs.py:63-70)."""
    from fem.cs import Axis
    rng = np.random.default_rng(8)
    normals = np.concatenate([np.eye(3), -np.eye(3), rng.normal(size=(10, 3)),
                              [[0.9995, 0.01, 0.0], [1.0, 1e-4, 0.0]]])
    bases = np.stack([Axis(n).construct_cs()._basis for n in normals])
    np.savez_compressed(os.path.join(HERE, "frames.npz"), normals=normals, bases=bases)
    print(f"frames: {len(normals)} normals")


def make_port_elements():
    from fem.physics.edm import nedeleclegrange2 as ref_nl
    rng = np.random.default_rng(77)
    n = 24
    verts = np.zeros((n, 2, 3))
    lem = np.zeros((n, 2, 3), dtype=np.int64)
    Ms = np.zeros((n, 3, 3), dtype=np.complex128)
    Mm = np.zeros((n, 3, 3), dtype=np.complex128)
    k0 = rng.uniform(100, 400, n)
    A = np.zeros((n, 14, 14), dtype=np.complex128)
    B = np.zeros((n, 14, 14), dtype=np.complex128)
    pairs = [(0, 1), (1, 2), (0, 2)]
    for k in range(n):
        h = 10 ** rng.uniform(-3.5, -2)
        v = rng.uniform(-1, 1, (2, 3)) * h + rng.uniform(-0.05, 0.05, (2, 1))
        verts[k] = v
        for e, (a, b) in enumerate(pairs):
            lem[k, :, e] = (a, b) if rng.random() < 0.5 else (b, a)
        Ms[k] = _rand_c3(rng, k % 3 == 0)
        Mm[k] = _rand_c3(rng, k % 3 == 0)
        A[k], B[k] = ref_nl.generalized_matrix_GQ(v, lem[k], Ms[k], Mm[k], float(k0[k]))
    np.savez_compressed(os.path.join(HERE, "port_elements.npz"), verts=verts, local_edge_map=lem, Ms=Ms, Mm=Mm,
                        k0=k0, A=A, B=B)
    print(f"port_elements: {n} triangles")


def dipole_surface(h=6e-3, half=0.03, k0=2 * np.pi * 10e9 / C0, seed=5):
    """A closed box surface around a z-directed short dipole at the origin.

    Returns (surface dict, Ein, Hin) with the surface arrays stratton_chu reads
    (n_tris, tri_to_edge, normals (outward), areas, edge_centers) and the dipole's
    E and H (unit current moment) at the edge centres; a few sources are scaled
    below sc.py's 1e-3 cut-off."""
    g = np.linspace(-half, half, int(round(2 * half / h)) + 1)
    tm = structured_box(g, g, g)
    tris = []
    normals = []
    for tag, nrm in ((pm.FACE_XMIN, (-1, 0, 0)), (pm.FACE_XMAX, (1, 0, 0)), (pm.FACE_YMIN, (0, -1, 0)),
                     (pm.FACE_YMAX, (0, 1, 0)), (pm.FACE_ZMIN, (0, 0, -1)), (pm.FACE_ZMAX, (0, 0, 1))):
        t = np.asarray(tm.boundary[tag], dtype=np.int64)
        tris.append(np.sort(t, axis=0))
        normals.append(np.repeat(np.array(nrm, dtype=float)[:, None], t.shape[1], axis=1))
    tris = np.concatenate(tris, axis=1)
    normals = np.concatenate(normals, axis=1)
    pairs = np.concatenate([tris[[0, 1]], tris[[1, 2]], tris[[0, 2]]], axis=1)
    key = pairs[0] * tm.n_nodes + pairs[1]
    ukey, inv = np.unique(key, return_inverse=True)
    tri_to_edge = inv.reshape(3, -1)
    ev = np.stack([ukey // tm.n_nodes, ukey % tm.n_nodes])
    centers = 0.5 * (tm.nodes[:, ev[0]] + tm.nodes[:, ev[1]])
    p0, p1, p2 = tm.nodes[:, tris[0]], tm.nodes[:, tris[1]], tm.nodes[:, tris[2]]
    areas = 0.5 * np.linalg.norm(np.cross((p1 - p0).T, (p2 - p0).T), axis=1)
    # short z dipole of unit current moment, e^{-jkr} convention (near + far terms):
    # H = jk g (1 + 1/(jkr)) z x r^,  E = eta g [2/r (1 + 1/(jkr)) cos(th) r^
    #     + jk (1 + 1/(jkr) - 1/(kr)^2) (cos(th) r^ - z)],  g = e^{-jkr} / (4 pi r)
    r = np.linalg.norm(centers, axis=0)
    rh = centers / r
    kr = k0 * r
    eta = 376.73031366857
    g0 = np.exp(-1j * kr) / (4 * np.pi * r)
    zhat = np.array([0.0, 0.0, 1.0])[:, None]
    cz = rh[2]
    a1 = 1 + 1 / (1j * kr)
    a2 = 1 + 1 / (1j * kr) - 1 / kr ** 2
    E = eta * g0 * (2 / r * a1 * cz * rh + 1j * k0 * a2 * (cz * rh - zhat))
    H = 1j * k0 * g0 * a1 * np.cross(zhat.T, rh.T).T
    rng = np.random.default_rng(seed)
    low = rng.choice(centers.shape[1], 25, replace=False)
    E[:, low] *= 1e-4
    H[:, low] *= 1e-4
    surf = dict(n_tris=tris.shape[1], tri_to_edge=tri_to_edge, normals=normals, areas=areas,
                edge_centers=centers)
    return surf, E, H


def make_farfield():
    """Reference Stratton-Chu far field of the dipole surface fields."""
    import types as _types
    from fem.physics.edm import sc as ref_sc
    k0 = 2 * np.pi * 10e9 / C0
    surf, E, H = dipole_surface(k0=k0)
    mesh = _types.SimpleNamespace(**surf)
    th = np.linspace(-np.pi / 2, np.pi / 2, 19)
    ph = np.linspace(0, 2 * np.pi, 36, endpoint=False)
    TH, PH = np.meshgrid(th, ph, indexing="ij")
    theta, phi = TH.ravel(), PH.ravel()
    t0 = time.time()
    Eout, Hout = ref_sc.stratton_chu(E, H, mesh, theta, phi, k0)
    print(f"farfield: {E.shape[1]} sources x {theta.size} directions ({time.time() - t0:.1f} s)")
    np.savez_compressed(os.path.join(HERE, "farfield.npz"), Ein=E, Hin=H, theta=theta, phi=phi, k0=k0,
                        Eout=Eout, Hout=Hout, **surf)


if __name__ == "__main__":
    which = _ARGS or ["tet", "tri", "small", "waveguide", "abc", "interp", "lumped", "frames", "port",
                      "farfield", "waveguide_k", "waveguide_diel", "port_interp"]
    if "tet" in which:
        make_tet_elements()
    if "tri" in which:
        make_tri_elements()
    if "small" in which:
        make_small_assembly()
    if "waveguide" in which:
        make_waveguide()
    if "abc" in which:
        make_waveguide_abc()
    if "interp" in which:
        make_interp()
    if "lumped" in which:
        make_lumped()
    if "frames" in which:
        make_frames()
    if "port" in which:
        make_port_elements()
    if "farfield" in which:
        make_farfield()
    if "waveguide_k" in which:
        make_waveguide_k()
    if "waveguide_diel" in which:
        make_waveguide_diel()
    if "port_interp" in which:
        make_port_interp()
