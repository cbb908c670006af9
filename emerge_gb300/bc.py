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
