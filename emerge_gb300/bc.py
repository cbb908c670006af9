"""Boundary conditions of the frequency-domain path (port and absorbing Robin terms, PEC).

These restate the coefficient functions of fem/bc.py that the assembler and the
sweep call per frequency; they are duck-type compatible with the reference's
classes (``tags``, ``get_gamma``, ``get_beta``, ``get_Uinc``, ``get_inv_basis``,
``cs.origin``, ``port_number``, ``_include_stiff`` / ``_include_force``), so the
GPU assembler accepts either.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

C0 = 299792458.0
ZVAC = 376.730313412


@dataclass
class CoordinateSystem:
    """Local frame (columns xax, yax, zax) and origin (fem/cs.py:221-247)."""
    xax: np.ndarray
    yax: np.ndarray
    zax: np.ndarray
    origin: np.ndarray

    def __post_init__(self):
        self.xax = np.asarray(self.xax, dtype=float)
        self.yax = np.asarray(self.yax, dtype=float)
        self.zax = np.asarray(self.zax, dtype=float)
        self.origin = np.asarray(self.origin, dtype=float)
        self._basis = np.array([self.xax, self.yax, self.zax]).T
        self._basis_inv = np.linalg.pinv(self._basis)

    def in_local_cs(self, x, y, z):
        p = self._basis_inv @ (np.array([x, y, z]) - self.origin[:, None])
        return p[0], p[1], p[2]

    def in_global_basis(self, x, y, z):
        v = self._basis @ np.array([x, y, z])
        return v[0], v[1], v[2]

    def in_global_cs(self, x, y, z):
        p = self._basis @ np.array([x, y, z]) + self.origin[:, None]
        return p[0], p[1], p[2]

    def in_local_basis(self, x, y, z):
        v = self._basis_inv @ np.array([x, y, z])
        return v[0], v[1], v[2]


class PEC:
    """Perfect electric conductor on the faces with the given tags (fem/bc.py:131-145)."""

    def __init__(self, tags):
        self.tags = list(tags)


class RectangularWaveguide:
    """TE_mn rectangular waveport (fem/bc.py:496-618), default TE10.

    gamma = j*beta, beta = sqrt(k0^2 - (pi m/w)^2 - (pi n/h)^2);
    U_inc = -2j*beta * E_mode, E_mode = A cos(pi m x/w) cos(pi n y/h) along local y,
    A = sqrt(4 * power * 377 / (w h)).
    """

    _include_stiff = True
    _include_mass = False
    _include_force = True
    modetype = "TEM"          # the reference's PortBC.modetype property (fem/bc.py:204-206)

    def __init__(self, tags, port_number: int, cs: CoordinateSystem, dims: tuple[float, float],
                 power: float = 1.0, mode: tuple[int, int] = (1, 0)):
        self.tags = list(tags)
        self.port_number = port_number
        self.cs = cs
        self.dims = dims
        self.power = power
        self.mode = mode
        self.active = False
        self.v_integration = False
        self.Z0 = None
        self.mode_number = 1

    def get_inv_basis(self):
        return self.cs._basis_inv

    def get_amplitude(self, k0):
        return np.sqrt(self.power * 4 * 377 / (self.dims[0] * self.dims[1]))

    def get_beta(self, k0):
        w, h = self.dims
        return np.sqrt(k0 ** 2 - (np.pi * self.mode[0] / w) ** 2 - (np.pi * self.mode[1] / h) ** 2)

    def get_gamma(self, k0):
        return 1j * self.get_beta(k0)

    def port_mode_3d(self, x_local, y_local, k0):
        w, h = self.dims
        E = self.get_amplitude(k0) * np.cos(np.pi * self.mode[0] * x_local / w) * np.cos(np.pi * self.mode[1] * y_local / h)
        return np.array([0 * E, E, 0 * E])

    def port_mode_3d_global(self, x, y, z, k0):
        xl, yl, _ = self.cs.in_local_cs(x, y, z)
        Ex, Ey, Ez = self.port_mode_3d(xl, yl, k0)
        return np.array(self.cs.in_global_basis(Ex, Ey, Ez))

    def get_Uinc(self, x_local, y_local, k0):
        return -2 * 1j * self.get_beta(k0) * self.port_mode_3d(x_local, y_local, k0)

    def Zmode(self, k0):
        return ZVAC


def _unit(v) -> np.ndarray:
    v = np.asarray(v, dtype=float)
    return v / np.linalg.norm(v)


def frame_from_normal(normal) -> CoordinateSystem:
    """The port frame the reference builds from a face normal (fem/cs.py:63-70):
    a = x unless the normal is within 0.999 of x (then y); yax = n x a,
    xax = -(n x yax), zax = n, origin 0; every vector normalised."""
    n = _unit(normal)
    a = np.array([1.0, 0.0, 0.0])
    if abs(np.dot(n, a)) > 0.999:
        a = np.array([0.0, 1.0, 0.0])
    y = _unit(np.cross(n, a))
    x = _unit(-np.cross(n, y))
    return CoordinateSystem(x, y, n, np.zeros(3))


class LumpedPort:
    """Lumped (sheet-impedance) port (fem/bc.py:620-745).

    A Robin boundary with sheet impedance Zs = Z0 w / h: gamma = j k0 376.7303 / Zs,
    U_inc = -2j k0 (V/h)(376.7303/Zs) d with the port voltage V = sqrt(2 P Z0) and the
    unit field direction d in the port frame.  The frame is built from the face
    normal as the reference does.  S-parameters use the voltage along a line of
    ``height`` in ``direction`` (``integration_line``, fem/physics/edm/emfreq3d.py:366-389).
    """

    _include_stiff = True
    _include_mass = False
    _include_force = True
    modetype = "TEM"
    ETA = 376.7303            # the literal of fem/bc.py:709,712

    def __init__(self, tags, port_number: int, width: float, height: float, direction, normal,
                 active: bool = False, power: float = 1.0, Z0: float = 50.0):
        self.tags = list(tags)
        self.port_number = port_number
        self.width = float(width)
        self.height = float(height)
        self.direction = _unit(direction)
        self.cs = frame_from_normal(normal)
        self.active = active
        self.power = float(power)
        self.Z0 = float(Z0)
        self.v_integration = True
        self.vintline = None

    @property
    def surfZ(self) -> float:
        return self.Z0 * self.width / self.height

    @property
    def voltage(self) -> float:
        return float(np.sqrt(2 * self.power * self.Z0))

    def get_inv_basis(self):
        return self.cs._basis_inv

    def get_beta(self, k0):
        return k0

    def get_gamma(self, k0):
        return 1j * k0 * self.ETA / self.surfZ

    def amplitude(self) -> float:
        """|U_inc| / (2 k0): the mode amplitude V/h * 376.7303/Zs."""
        return self.voltage / self.height * (self.ETA / self.surfZ)

    def port_mode_3d(self, x_local, y_local, k0):
        B = self.cs._basis_inv
        d = self.direction
        p = B @ d
        one = np.ones_like(np.asarray(x_local, dtype=float))
        return np.array([p[0] * one, p[1] * one, p[2] * one])

    def port_mode_3d_global(self, x, y, z, k0):
        xl, yl, _ = self.cs.in_local_cs(x, y, z)
        Ex, Ey, Ez = self.port_mode_3d(xl, yl, k0)
        return np.array(self.cs.in_global_basis(Ex, Ey, Ez))

    def get_Uinc(self, x_local, y_local, k0):
        Emag = -1j * 2 * k0 * self.voltage / self.height * (self.ETA / self.surfZ)
        return Emag * self.port_mode_3d(x_local, y_local, k0)

    def integration_line(self, mesh, n_points: int = 11):
        """Voltage line of the port (fem/physics/edm/emfreq3d.py:366-389, fem/coord.py:21-52):
        from the mean of the port-face nodes of least coordinate along ``direction``,
        ``height`` along it, ``n_points`` points; returns (midpoints (3, n-1), steps (3, n-1))."""
        tri = np.asarray(mesh.get_triangles(self.tags), dtype=np.int64)
        pts = np.unique(np.asarray(mesh.tris)[:, tri].ravel())
        nodes = np.asarray(mesh.nodes)
        d = self.direction
        dot = nodes[0, pts] * d[0] + nodes[1, pts] * d[1] + nodes[2, pts] * d[2]
        start = np.mean(nodes[:, pts[dot == np.min(dot)]], axis=1)
        end = start + d * self.height
        xs = [np.linspace(start[c], end[c], n_points) for c in range(3)]
        mid = np.array([0.5 * (x[:-1] + x[1:]) for x in xs])
        step = np.array([x[1:] - x[:-1] for x in xs])
        return mid, step


class AbsorbingBoundary:
    """First-order absorbing boundary (fem/bc.py:254-300): gamma = j*k0, no forcing."""

    _include_stiff = True
    _include_mass = True
    _include_force = False

    def __init__(self, tags):
        self.tags = list(tags)

    def get_beta(self, k0):
        return k0

    def get_gamma(self, k0):
        return 1j * k0


def is_pec(bc) -> bool:
    return type(bc).__name__ == "PEC"


def is_robin(bc) -> bool:
    return hasattr(bc, "_include_stiff") and hasattr(bc, "get_gamma")


def is_port(bc) -> bool:
    return is_robin(bc) and hasattr(bc, "port_number") and bool(getattr(bc, "_include_force", False))


@dataclass
class PortMode:
    """One solved mode of a ModalPort (fem/bc.py:302-327): the surface field, its
    propagation constant, normalisation and type."""
    modefield: np.ndarray            # (n_field,) complex, the port surface's numbering
    k0: float
    beta: float
    freq: float
    norm_factor: float = 1.0
    TEM: bool = False
    modetype: str = "TEM"
    energy: float = 0.0
    power: float = 0.0               # the integrated power flux before normalisation
    Z0: float | None = None

    @property
    def neff(self) -> float:
        return self.beta / self.k0


class ModalPort:
    """Waveport whose mode comes from a 2-D eigen solve of the port face
    (fem/bc.py:329-494 ModalPort with the post-processing of
    Electrodynamics3D.modal_analysis, fem/physics/edm/emfreq3d.py:201-365).

    ``modal_analysis`` solves the port problem on the GPU (``modes.port_problem``, the
    dense eigensolve, the reference's mode filter), then per mode: the phase is turned
    so the largest entry (numpy's complex max) is real, beta = min(sqrt(-lambda), kmax),
    the integrated power flux 0.5 Re(E x H*) . n of the mode over the face gives
    norm_factor = 1/sqrt(|P|), modes with mean |field|^2 below 1e-4 are dropped, and
    TE / TM follows from max|E_z| / max|E_t| < 1e-5.  The fields are evaluated by the
    GPU interpolation of the Nedelec-Lagrange-2 basis (``emg_port_interp``).
    TEM ports (conductor detection and the voltage line of modal_analysis) are not built.
    """

    _include_stiff = True
    _include_mass = False
    _include_force = True

    def __init__(self, tags, port_number: int, cs: CoordinateSystem | None = None, power: float = 1.0,
                 active: bool = False, normal=None):
        self.tags = list(tags)
        self.port_number = port_number
        self.power = power
        self.active = active
        if cs is None:
            if normal is None:
                raise ValueError("ModalPort: give cs or the face normal")
            cs = frame_from_normal(normal)
        self.cs = cs
        self.selected_mode = 0
        self.modes: list[PortMode] = []
        self.v_integration = False
        self.Z0 = None
        self.mode_number = 1
        self._surface = None

    # ------------------------------------------------------------- the solve ---
    def modal_analysis(self, field, er, ur, freq: float, pec_tags=(), nmodes: int | None = None,
                       target_kz: float | None = None, face_block: bool = False, device="cuda") -> list[PortMode]:
        """Solve the port face's modes at ``freq`` and store them (emfreq3d.py:201-365)."""
        import torch
        from .assembly import matinv_device
        from .modes import port_field, port_problem
        k0 = 2 * np.pi * freq / C0
        m = field.mesh
        dev = torch.device(device)
        pp = port_problem(field, er, ur, self.tags, self.cs._basis, k0, pec_tags, target_kz, face_block, device)
        S = pp.surface
        sid = torch.as_tensor(pp.solve_ids, device=dev)
        t = pp.target_kz
        sigma = -t * t
        mu, vec = torch.linalg.eig(torch.linalg.solve(pp.A - sigma * pp.B, pp.B))
        mu = mu.cpu().numpy()
        lam = np.full(mu.shape, np.inf + 0j)
        finite = np.abs(mu) > 1e-12 * np.abs(mu).max()
        lam[finite] = sigma + 1.0 / mu[finite]
        keep = np.flatnonzero((lam.real <= -1) & (lam.real >= -(t ** 2) * 8))
        keep = keep[np.argsort(np.abs(np.sqrt(-lam[keep]) - t))]
        if nmodes is not None:
            keep = keep[:nmodes]
        tri_ids = np.asarray(m.get_triangles(self.tags), dtype=np.int64)
        tet_of = np.asarray(m.tri_to_tet)[0, tri_ids]
        er_t = np.asarray(er)[:, :, tet_of]
        ur_t = np.asarray(ur)[:, :, tet_of]
        kmax = k0 * np.sqrt(np.max(er_t.ravel()) * np.max(ur_t.ravel()))
        urinv = matinv_device(torch.as_tensor(np.ascontiguousarray(ur_t.reshape(9, -1)), device=dev))
        urinv_diag = urinv[[0, 4, 8]].contiguous()
        nodes = np.asarray(m.nodes)[:, S.node_ids]
        xl, yl, _ = self.cs.in_local_cs(nodes[0], nodes[1], nodes[2])
        self._surface = (S, np.stack([xl, yl]), urinv_diag)
        from .freq import dunavant6
        D = dunavant6()
        v1, v2, v3 = nodes[:, S.tris[0]], nodes[:, S.tris[1]], nodes[:, S.tris[2]]
        nrm = np.cross((v2 - v1).T, (v3 - v1).T)
        area = np.linalg.norm(nrm, axis=1) / 2
        n0 = nrm[0] / np.linalg.norm(nrm[0])
        pts = np.concatenate([v1 * D[1, k] + v2 * D[2, k] + v3 * D[3, k] for k in range(D.shape[1])], axis=1)
        self.modes = []
        for i in keep:
            E = torch.zeros(S.n_field, dtype=torch.complex128, device=dev)
            E[sid] = vec[:, int(i)]
            Eh = E.cpu().numpy()
            big = Eh[np.lexsort((Eh.imag, Eh.real))[-1]]             # numpy's complex max
            E = E * np.exp(-1j * np.angle(big))
            beta = min(np.emath.sqrt(-lam[i]).real, kmax.real)
            Eg = self._eval(E, pts, 0, 0.0)
            Hg = self._eval(E, pts, 1, beta) * (1j / ((k0 * C0) * (4 * np.pi * 1e-7)))
            Sv = 0.5 * np.real(np.cross(Eg.T, np.conj(Hg).T)) @ n0
            P = 0.0
            npt = S.tris.shape[1]
            for k in range(D.shape[1]):
                P += D[0, k] * np.sum(Sv[k * npt:(k + 1) * npt] * area)
            Ehost = E.cpu().numpy()
            energy = float(np.mean(np.abs(Ehost) ** 2))
            if energy < 1e-4:
                continue
            mode = PortMode(Ehost, k0, float(beta), freq, norm_factor=float(np.sqrt(1 / np.abs(P))),
                            energy=energy, power=float(P))
            ez = np.max(np.abs(Ehost[S.n_xy:]))
            exy = np.max(np.abs(Ehost[:S.n_xy]))
            mode.modetype = "TE" if ez / exy < 1e-5 else "TM"
            self.modes.append(mode)
        return self.modes

    def _eval(self, E, pts_global, which: int, beta: float) -> np.ndarray:
        """The mode's E (which 0) or curl term (which 1) at global points, global basis."""
        from .modes import port_field
        S, nodes_local, urinv_diag = self._surface
        xl, yl, _ = self.cs.in_local_cs(pts_global[0], pts_global[1], pts_global[2])
        loc = port_field(S, nodes_local, E, np.stack([xl, yl]), which, urinv_diag, beta)
        return np.array(self.cs.in_global_basis(loc[0], loc[1], loc[2]))

    # ------------------------------------------------- the port's coefficients ---
    @property
    def modetype(self) -> str:
        return self.get_mode().modetype

    def get_mode(self, i=None) -> PortMode:
        return self.modes[self.selected_mode if i is None else i]

    def get_inv_basis(self):
        return self.cs._basis_inv

    def get_beta(self, k0):
        """beta(k0) from the solved mode (fem/bc.py:444-453)."""
        mode = self.get_mode()
        if mode.TEM:
            return mode.beta / mode.k0 * k0
        freq = k0 * C0 / (2 * np.pi)
        return np.sqrt(mode.beta ** 2 + k0 ** 2 * (1 - ((mode.freq / freq) ** 2)))

    def get_gamma(self, k0):
        return 1j * self.get_beta(k0)

    def port_mode_3d_global(self, x, y, z, k0):
        import torch
        mode = self.get_mode()
        E = torch.as_tensor(mode.modefield, device=self._surface[2].device)
        Eg = self._eval(E, np.array([np.atleast_1d(x), np.atleast_1d(y), np.atleast_1d(z)], dtype=float), 0, 0.0)
        return np.sqrt(self.power) * mode.norm_factor * Eg

    def port_mode_3d(self, x_local, y_local, k0):
        xg, yg, zg = self.cs.in_global_cs(np.asarray(x_local), np.asarray(y_local), 0 * np.asarray(x_local))
        Eg = self.port_mode_3d_global(xg, yg, zg, k0)
        return np.array(self.cs.in_local_basis(Eg[0], Eg[1], Eg[2]))

    def get_Uinc(self, x_local, y_local, k0):
        return -2 * 1j * self.get_beta(k0) * self.port_mode_3d(x_local, y_local, k0)

    def Zmode(self, k0):
        """PortBC.Zmode (fem/bc.py:207-215)."""
        kind = self.modetype
        if kind == "TE":
            return k0 * C0 / self.get_beta(k0) * 4 * np.pi * 1e-7
        if kind == "TM":
            return self.get_beta(k0) / (k0 * C0 * 8.854187818814e-12)
        return ZVAC
