"""CPU oracle for the angular-spectrum propagation path of lightprop2d 1.0.4.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the CUDA backend in
``lightprop2d_gb300`` never imports it.  Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline leg of ``bench.py`` may use it.

It restates, in plain numpy (float64 / complex128 unless told otherwise), the
reference's own algorithm so that every GPU result can be compared with it:

* grids ............ lightprop2d/beam2d.py:299-308 (``_construct_grids``) and
                     :189-205 (``_k_grid`` -> ``fftfreq``)
* fft2 / ifft2 ..... lightprop2d/beam2d.py:207-229 (numpy convention: the inverse
                     carries the 1/N^2 factor)
* propagate ........ lightprop2d/beam2d.py:481-490
* lens ............. lightprop2d/beam2d.py:508-511
* coordinate_filter  lightprop2d/beam2d.py:335-342
* spectral_filter .. lightprop2d/beam2d.py:366-373
* iprofile ......... lightprop2d/beam2d.py:717-721

Parity is pinned: ``tests/test_oracle.py`` checks this module against golden
vectors produced by running the reference itself (``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import numpy as np

nm = 1e-7
um = 1e-4
mm = 1e-1
cm = 1
m = 100


def grids(area_size: float, npoints: int, wl: float) -> dict:
    """Grids exactly as ``Beam2D._construct_grids`` builds them (beam2d.py:299-308).

    X is a centred row vector, Y its column; Kx = fftfreq(N, dL) is unshifted
    and in cycles/cm; Kz = nan_to_num(sqrt(k0^2 - Kx^2 - Ky^2)) so evanescent
    entries become 0 (a pass-through of the transfer function, not a mask).
    """
    dL = area_size / npoints
    X = np.arange(-npoints // 2, npoints // 2, 1) * dL
    Y = X.reshape((-1, 1))
    k0 = 1 / wl
    Kx = np.fft.fftfreq(npoints, d=dL)
    Ky = Kx.reshape((-1, 1))
    with np.errstate(invalid="ignore"):
        Kz = np.nan_to_num(np.sqrt(k0 ** 2 - Kx ** 2 - Ky ** 2))
    return dict(dL=dL, X=X, Y=Y, k0=k0, Kx=Kx, Ky=Ky, Kz=Kz)


def fft2(a: np.ndarray) -> np.ndarray:
    """beam2d.py:217 (numpy path): unnormalised forward 2-D DFT."""
    return np.fft.fft2(a)


def ifft2(a: np.ndarray) -> np.ndarray:
    """beam2d.py:229 (numpy path): inverse 2-D DFT with the 1/N^2 factor."""
    return np.fft.ifft2(a)


def transfer(Kz: np.ndarray, z: float) -> np.ndarray:
    """exp(i*phase) with phase = 2*pi*(trunc(Kz*z) - Kz*z), beam2d.py:485-489."""
    dk = Kz * z
    phase = 2 * np.pi * (np.trunc(dk) - dk)
    return np.cos(phase) + 1j * np.sin(phase)


def propagate(spectrum: np.ndarray, Kz: np.ndarray, z: float):
    """``Beam2D.propagate`` body (beam2d.py:481-490).

    Returns (spectrum_new, field_new).  ``z == 0`` is a no-op in the reference
    (returns before touching anything); callers handle that case.  The in-place
    ``*=`` of the reference casts the complex128 transfer function into the
    spectrum's dtype, which ``np.multiply(..., out=)`` reproduces.
    """
    s = spectrum.copy()
    np.multiply(s, transfer(Kz, z), out=s, casting="same_kind")
    return s, ifft2(s)


def lens_phase(X: np.ndarray, Y: np.ndarray, k0: float, f: float) -> np.ndarray:
    """exp(i*(X^2+Y^2)*k0/(2f)) as built in beam2d.py:508-510 (k0 = 1/wl, no 2*pi)."""
    phase = (X ** 2 + Y ** 2) * k0 / (2 * f)
    return np.cos(phase) + 1j * np.sin(phase)


def lens(field: np.ndarray, X, Y, k0: float, f: float):
    """``Beam2D.lens`` body (beam2d.py:508-511): returns (field_new, spectrum_new)."""
    fl = field.copy()
    np.multiply(fl, lens_phase(X, Y, k0, f), out=fl, casting="same_kind")
    return fl, fft2(fl)


def coordinate_filter(field: np.ndarray, mask: np.ndarray):
    """``Beam2D.coordinate_filter`` with an array mask (beam2d.py:339-342)."""
    fl = field.copy()
    np.multiply(fl, mask, out=fl, casting="same_kind")
    return fl, fft2(fl)


def spectral_filter(spectrum: np.ndarray, mask: np.ndarray):
    """``Beam2D.spectral_filter`` with an array mask (beam2d.py:370-373)."""
    s = spectrum.copy()
    np.multiply(s, mask, out=s, casting="same_kind")
    return s, ifft2(s)


def iprofile(field: np.ndarray) -> np.ndarray:
    """|field|^2 (beam2d.py:717)."""
    return np.abs(field) ** 2


class OracleBeam:
    """Stateful restatement of ``Beam2D`` for the propagation path.

    Holds (field, spectrum, z) like the reference dataclass (beam2d.py:79-133):
    the spectrum is state, ``propagate`` multiplies it in place and overwrites
    the field; ``lens`` / ``coordinate_filter`` overwrite the spectrum.
    """

    def __init__(self, area_size, npoints, wl, init_field=None,
                 init_spectrum=None, complex_bits=128):
        g = grids(area_size, npoints, wl)
        self.area_size, self.npoints, self.wl = area_size, npoints, wl
        self.__dict__.update(g)
        self.complex = np.complex64 if complex_bits == 64 else np.complex128
        if init_field is None:
            raise ValueError("init_field is required")
        self.field = np.asarray(init_field).astype(self.complex)
        self.spectrum = (fft2(self.field) if init_spectrum is None
                         else np.asarray(init_spectrum))
        self.z = 0.0

    def propagate(self, z):
        if z == 0:
            return
        self.z += z
        self.spectrum, self.field = propagate(self.spectrum, self.Kz, z)

    def lens(self, f):
        self.field, self.spectrum = lens(self.field, self.X, self.Y, self.k0, f)

    def coordinate_filter(self, mask):
        self.field, self.spectrum = coordinate_filter(self.field, mask)

    def spectral_filter(self, mask):
        self.spectrum, self.field = spectral_filter(self.spectrum, mask)

    @property
    def iprofile(self):
        return iprofile(self.field)


# --------------------------------------------------------------------------
# Error metrics used by every parity test.
# --------------------------------------------------------------------------

def rel_l2(a, b) -> float:
    """||a - b||_2 / ||b||_2 in float64 (b is the oracle)."""
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    nb = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (nb if nb > 0 else 1.0))


def energy_err(a, b) -> float:
    """|sum|a|^2 - sum|b|^2| / sum|b|^2 (energy conservation vs the oracle)."""
    ea = float(np.sum(np.abs(np.asarray(a, dtype=np.complex128)) ** 2))
    eb = float(np.sum(np.abs(np.asarray(b, dtype=np.complex128)) ** 2))
    return abs(ea - eb) / (eb if eb > 0 else 1.0)


# --------------------------------------------------------------------------
# Seeded input builders for the benchmark / parity workloads.  They compose
# the reference's generators (profiles.py) the way each workload describes.
# --------------------------------------------------------------------------

def random_phase_hole(npoints, area_size, radius, seed):
    """Round hole of geometric radius ``radius`` (r <= radius), amplitude
    U[0,1) and phase 2*pi*U[0,1) from ``np.random.default_rng(seed)``, zero
    outside.  Used for the 256^2 / 200 um / 632 nm CPU workload.
    """
    g = grids(area_size, npoints, 1.0)
    rng = np.random.default_rng(seed)
    amp = rng.uniform(size=(npoints, npoints))
    ph = rng.uniform(size=(npoints, npoints))
    r2 = g["X"] ** 2 + g["Y"] ** 2
    f = amp * np.exp(2j * np.pi * ph)
    f[r2 > radius ** 2] = 0
    return f


def gaussian(npoints, area_size, A0, rho0):
    """profiles.gaussian_beam (profiles.py:64-71) on the Beam2D grid."""
    g = grids(area_size, npoints, 1.0)
    return A0 * np.exp(-(g["X"] ** 2 + g["Y"] ** 2) / rho0 ** 2)


def gaussian_paraxial(npoints, area_size, wl, rho0, z):
    """Analytic paraxial propagation of ``gaussian(npoints, area_size, 1,
    rho0)`` by z (the known answer of config 2 and of the reference's
    tests/test_analytics.py:53-71): with k = 2*pi/wl, z_R = k*rho0^2/2,
    q = z + i*z_R, E = (i*z_R/q) * exp(-i*k*r^2/(2q)) * exp(-i*k*z).  The
    angular-spectrum result departs from it by the non-paraxial terms
    (~2.5e-7 rel-L2 per cm at 2 mm / 2048^2 / 632 nm / 100 um) until the beam
    wraps in the periodic window."""
    g = grids(area_size, npoints, wl)
    k = 2 * np.pi / wl
    zr = k * rho0 ** 2 / 2
    q0 = 1j * zr
    q = q0 + z
    return (q0 / q) * np.exp(-1j * k * (g["X"] ** 2 + g["Y"] ** 2) / (2 * q)) * np.exp(-1j * k * z)


# --------------------------------------------------------------------------
# Beam metrics and grid management (beam2d.py:375-460, :669-752).
# --------------------------------------------------------------------------

def centroid(field, dL):
    """``Beam2D.centroid`` (beam2d.py:669-685): (Xc, Yc, nxc, nyc)."""
    n = field.shape[0] // 2
    Y, X = np.mgrid[-n:n, -n:n] * dL
    I = np.abs(field) ** 2
    Xc = np.average(X, weights=I)
    Yc = np.average(Y, weights=I)
    return Xc, Yc, int(Xc / dL) + n, int(Yc / dL) + n


def d4sigma(field, dL):
    """``Beam2D.D4sigma`` (beam2d.py:687-704): 4*sigma along x and y."""
    n = field.shape[0] // 2
    I = np.abs(field) ** 2
    Y, X = np.mgrid[-n:n, -n:n] * dL
    Xc, Yc, _, _ = centroid(field, dL)
    return (4 * np.sqrt(np.average((X - Xc) ** 2, weights=I)),
            4 * np.sqrt(np.average((Y - Yc) ** 2, weights=I)))


def centroid_intensity(field, dL):
    """``Beam2D.centroid_intensity`` (beam2d.py:740-752)."""
    _, _, nxc, nyc = centroid(field, dL)
    return float(np.abs(field[nyc, nxc]) ** 2)


def expand(field, n_out):
    """``Beam2D.expand`` field step (beam2d.py:390-402): pad (n_out - n)/2
    points on every side with copies of the edge rows/columns."""
    d = (n_out - field.shape[0]) // 2
    return np.pad(field, d, mode="edge")


def coarse(field, order):
    """``Beam2D.coarse`` field step (beam2d.py:455-459): block mean."""
    n = field.shape[0] // order
    return field.reshape((n, order, n, order)).mean((1, 3))


def bilinear_nearest(grid_x, values, qx):
    """2-D linear interpolation of ``values`` (rows and columns on the
    ascending axis ``grid_x``) at the ascending query axis ``qx`` for both
    dimensions, nearest value outside the axis range.  This is what the
    reference's ``scipy.interpolate.interp2d(x, x, z)`` (kind="linear",
    fill_value=None) returns on a rectangular grid; interp2d itself was
    removed from SciPy 1.14, so it is restated here."""
    qx = np.sort(np.asarray(qx, dtype=np.float64))
    p = np.interp(qx, grid_x, np.arange(len(grid_x), dtype=np.float64))
    i0 = np.clip(np.floor(p).astype(int), 0, len(grid_x) - 1)
    i1 = np.minimum(i0 + 1, len(grid_x) - 1)
    w = p - i0
    v = np.asarray(values)
    rows = v[i0, :] * (1 - w)[:, None] + v[i1, :] * w[:, None]
    return rows[:, i0] * (1 - w)[None, :] + rows[:, i1] * w[None, :]


def crop(field, X, area_size, npoints_out, area_out):
    """``Beam2D.crop`` field step (beam2d.py:417-430): the central window
    |X| < area_size/2 resampled onto the new centred grid."""
    nc = field.shape[0] // 2
    n = len(X[np.abs(X) < area_size / 2]) // 2
    old_x = X[nc - n:nc + n]
    win = field[nc - n:nc + n, nc - n:nc + n]
    new_x = np.arange(-npoints_out // 2, npoints_out // 2, 1) * (area_out / npoints_out)
    return bilinear_nearest(old_x, win, new_x)


def lens_image(field, X, k0, l1, l2):
    """``Beam2D.lens_image`` field step (beam2d.py:524-535): the field
    resampled at the sorted coordinates s*X (s = -l1/l2), times s and the
    phase -(X^2+Y^2)*k0*(l1+l2)/(2*l2^2)."""
    s = -l1 / l2
    Y = X.reshape((-1, 1))
    phase = -(X ** 2 + Y ** 2) * k0 * (l1 + l2) / 2 / l2 ** 2
    g = bilinear_nearest(X, field, X * s)
    return s * g * (np.cos(phase) + 1j * np.sin(phase))


# --------------------------------------------------------------------------
# Mode decomposition (beam2d.py:539-667).
# --------------------------------------------------------------------------

def _window(field, nb):
    n = field.shape[0]
    d = (n - nb) // 2
    return field[d:n - d, d:n - d].flatten()


def modes_scalar(field, modes):
    """deconstruct_by_modes(mode="scalar") (beam2d.py:593-596): modes @ window."""
    modes = np.asarray(modes)
    nb = int(np.sqrt(modes.shape[1]))
    return np.vstack(modes) @ _window(field, nb)


def modes_lstsq(field, modes):
    """deconstruct_by_modes(mode="lstsq") (beam2d.py:597-599)."""
    modes = np.asarray(modes)
    nb = int(np.sqrt(modes.shape[1]))
    return np.linalg.lstsq(np.vstack(modes).T, _window(field, nb), rcond=-1)[0]


def modes_fast(field, modes_matrix_t, modes_matrix_dot_t):
    """fast_deconstruct_by_modes (beam2d.py:639-648)."""
    nb = int(np.sqrt(modes_matrix_t.shape[1]))
    return np.linalg.lstsq(modes_matrix_dot_t, modes_matrix_t.dot(_window(field, nb)),
                           rcond=None)[0]


def modes_combine(modes, coeffs, n):
    """construct_by_modes with _expand_basis (beam2d.py:539-559, :662-666)."""
    modes = np.asarray(modes)
    nb = int(np.sqrt(modes.shape[1]))
    d = (n - nb) // 2
    out = np.zeros((n, n), dtype=np.complex128)
    out[d:n - d, d:n - d] = np.einsum("ij,i->j", modes, coeffs).reshape(nb, nb)
    return out
