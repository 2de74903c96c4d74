"""FP64 NumPy background inverse of the 3D 27-point operator (oracle; tests only).

Checker for ``bella_spectral3d_apply``.  The operator of ``lap3D``
(laplacian.py:898-1026, restated in oracle/nodal3d.py) with every cell
coefficient replaced by its mean over the interior x and z cells per y-cell,
and ``hcenter`` by its mean per y-node, is a sum of Kronecker products of 1D
node operators.  Along a periodic axis (n nodes, period n-1, duplicated seam)
the difference form D^T D and the sum form M^T M are circulant and share the
Fourier eigenvectors; along a wall axis (outer cell planes zeroed) they share
the DCT-I eigenvectors cos(pi k i/(n-1)) with trapezoid weights.  Along y
(walls) the forms with the y-dependent means are tridiagonal.  This module
builds the exact background inverse with numpy FFTs along periodic axes,
dense DCT-I matrices along wall axes and a dense pseudo-inverse per (kx, kz)
line -- independent of the device method's Hartley GEMMs and pinned Thomas
solves.  Pinned by tests/test_oracle_3d.py: with coefficients that equal
their horizontal means, A (M r) = r for every r in the range of A.
The reference has no preconditioner (second_projection.py:230); nothing of
it is restated here beyond the operator.
"""
import numpy as np


def _line_forms(C):
    """D^T C D and M^T C M on n = len(C)+1 nodes, C on the cells between them."""
    n = len(C) + 1
    TD = np.zeros((n, n))
    TM = np.zeros((n, n))
    for c, v in enumerate(C):
        i, j = c, c + 1
        TD[i, i] += v; TD[j, j] += v; TD[i, j] -= v; TD[j, i] -= v
        TM[i, i] += v; TM[j, j] += v; TM[i, j] += v; TM[j, i] += v
    return TD, TM


def _axis(n, periodic):
    """(mu, forward(R, axis), inverse(X, axis)) of one axis."""
    if periodic:
        N = n - 1
        mu = 4.0 * np.sin(np.pi * np.arange(N) / N) ** 2

        def fwd(R, axis):
            R = np.moveaxis(R, axis, 0)
            P = R[:-1].copy()
            P[0] = 0.5 * (R[0] + R[-1])
            return np.moveaxis(np.fft.fft(P, axis=0), 0, axis)

        def inv(X, axis):
            X = np.moveaxis(X, axis, 0)
            P = np.fft.ifft(X, axis=0)
            return np.moveaxis(np.concatenate([P, P[:1]], axis=0), 0, axis)
    else:
        M = n - 1
        k = np.arange(n)
        mu = 4.0 * np.sin(0.5 * np.pi * k / M) ** 2
        V = np.cos(np.pi * np.outer(np.arange(n), k) / M)         # V[i, k]
        nrm = np.full(n, 0.5 * M)
        nrm[0] = nrm[-1] = M

        def fwd(R, axis):
            R = np.moveaxis(R, axis, -1)
            return np.moveaxis((R @ V) / nrm, -1, axis)

        def inv(X, axis):
            X = np.moveaxis(X, axis, -1)
            return np.moveaxis(X @ V.T, -1, axis)
    return mu, fwd, inv


class BackgroundInverse:
    """A_bg^+ for an operator packed by :func:`oracle.nodal3d.pack_27pt` (y must be a wall axis)."""

    def __init__(self, op):
        nx, ny, nz = op["nx"], op["ny"], op["nz"]
        walls = op["walls"]
        if not walls[1]:
            raise ValueError("the background inverse needs walls in y")
        self.shape = (nx, ny, nz)
        shp = (nx + 1, ny + 1, nz + 1)
        means = []
        for key in ("hplusx", "hplusy", "hplusz"):
            h = op[key].reshape(shp)
            means.append(h[1:nx, 1:ny, 1:nz].mean(axis=(0, 2)))       # interior y cells 1..ny-1
        hc = op["hcenter"].reshape(nx, ny, nz).mean(axis=(0, 2))
        TDx, TMx = _line_forms(means[0])
        TDy, TMy = _line_forms(means[1])
        TDz, TMz = _line_forms(means[2])
        mux, self.fx, self.ix = _axis(nx, not walls[0])
        muz, self.fz, self.iz = _axis(nz, not walls[2])
        dx2, dy2, dz2 = op["dx"] ** 2, op["dy"] ** 2, op["dz"] ** 2
        mx = mux[:, None, None, None]
        mz = muz[None, :, None, None]
        K = -(1.0 / 16.0) * ((mx * (4 - mz) / dx2) * TMx + ((4 - mx) * (4 - mz) / dy2) * TDy
                             + ((4 - mx) * mz / dz2) * TMz) + np.diag(hc)
        self.Kinv = np.linalg.pinv(K, rcond=1e-12, hermitian=True)    # (Kx, Kz, ny, ny)
        self.D = 1.0 / op["diag_inv"]

    def apply(self, r):
        """A_bg^+ (r / diag_inv) for a residual r of the Jacobi-scaled system (flat, C order)."""
        nx, ny, nz = self.shape
        R = (np.asarray(r, np.float64) * self.D).reshape(nx, ny, nz)
        Rh = self.fx(self.fz(R.astype(complex), 2), 0)                 # (Kx, ny, Kz)
        Xh = np.einsum("xkab,xbk->xak", self.Kinv, Rh)
        X = self.iz(self.ix(Xh, 0), 2)
        return np.real(X).reshape(-1)
