"""FP64 NumPy background inverse of the 2D 9-point operator (oracle; tests only).

Checker for ``bella_spectral2d_create`` + ``bella_spectral3d_apply``.  The
operator of ``lap2D_gather_new`` (laplacian.py:546-746, restated in
oracle/nodal2d.py) is, without the Coriolis cross terms,
  A = -1/4 [ (1/dx^2) (D_x^T D_x) (x) (M_y^T Cx M_y) + (1/dy^2) (M_x^T M_x) (x) (D_y^T Cy D_y) ] + hcenter
with Cx = cxx*hplusx and Cy = cyy*hplusy on the cells (D: differences, M: sums
of the two nodes of a cell).  With Cx, Cy replaced by their means over the
interior x cells per y-cell row and hcenter by its mean per node row, the
x-factors share the Fourier (periodic, duplicated seam averaged in and copied
out) or DCT-I (walls) eigenvectors with eigenvalues mu and 4 - mu, and every x
mode leaves a tridiagonal operator along y:
  K(mu) = -1/4 [ mu/dx^2 M_y^T Cx M_y + (4 - mu)/dy^2 D_y^T Cy D_y ] + diag(hcm).
This module inverts it with numpy FFTs / a dense DCT-I and a dense
pseudo-inverse per line.  Pinned by tests/test_oracle_golden.py: with
coefficients that equal their horizontal means and no cross terms,
A (M r) = r for every r in the range of A.
"""
import numpy as np

from oracle.spectral3d import _axis, _line_forms


class BackgroundInverse2D:
    """A_bg^+ for an operator packed by :func:`oracle.nodal2d.pack_9pt` (y must be a wall axis)."""

    def __init__(self, op):
        nx, ny = op["nx"], op["ny"]
        if not op["y_wall"]:
            raise ValueError("the background inverse needs walls in y")
        self.shape = (ny, nx)
        shp = (ny + 1, nx + 1)
        cxx, cyy = op["cor"][0], op["cor"][1]
        Cx = (np.asarray(cxx).reshape(shp) * op["hplusx"].reshape(shp))[1:ny, 1:nx].mean(axis=1)
        Cy = (np.asarray(cyy).reshape(shp) * op["hplusy"].reshape(shp))[1:ny, 1:nx].mean(axis=1)
        hc = op["hcenter"].reshape(ny, nx).mean(axis=1)
        _, TMx = _line_forms(Cx)
        TDy, _ = _line_forms(Cy)
        mu, self.fx, self.ix = _axis(nx, not op["x_wall"])
        m = mu[:, None, None]
        K = -0.25 * ((m / op["dx"] ** 2) * TMx + ((4 - m) / op["dy"] ** 2) * TDy) + np.diag(hc)
        self.Kinv = np.linalg.pinv(K, rcond=1e-12, hermitian=True)        # (Kx, ny, ny)
        self.D = 1.0 / op["diag_inv"]

    def apply(self, r):
        """A_bg^+ (r / diag_inv) for a residual r of the Jacobi-scaled system (flat, y-major)."""
        ny, nx = self.shape
        R = (np.asarray(r, np.float64) * self.D).reshape(ny, nx)
        Rh = self.fx(R.astype(complex), 1)                                 # (ny, Kx)
        Xh = np.einsum("kab,bk->ak", self.Kinv, Rh)
        return np.real(self.ix(Xh, 1)).reshape(-1)
