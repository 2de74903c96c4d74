"""Drop-in for the operator factory of the reference's ``laplacian`` module.

``stencil_9pt_numba_test`` keeps the reference's signature and operand
packing (laplacian.py:496-528) and returns a device operator instead of a
closure over the Numba kernel ``lap2D_gather_new`` (laplacian.py:546-746).
When ``ud`` has a ``LAMB_BDRY`` attribute (any value: the reference tests
``hasattr``, laplacian.py:511) it is the operator of the reference's other
closure, ``lap2D_numba_test`` with the ``kernel_9pt`` stencil
(laplacian.py:531-543, 749-868): the same operands, x periodic, y padded by
mirroring, no boundary cell zeroed.
"""
from .linalg import NodalHelmholtz2D

_WALLS = ("symmetric", "radiation")   # BdryType.WALL / BdryType.RAYLEIGH values (options.py:42-49)


def _is_wall(bt):
    v = getattr(bt, "value", bt)
    return v in _WALLS or str(v).lower() in ("wall", "rayleigh")


def stencil_9pt_numba_test(mpv, node, coriolis, diag_inv, ud, device=None):
    """Return the 2D nodal Helmholtz operator of one projection (laplacian.py:496-528).

    ``coriolis`` is the transposed 4-tuple of ``multiply_inverse_coriolis(...,
    get_coeffs=True)`` (second_projection.py:651); ``diag_inv`` the node.isc
    array from ``precon_diag_prepare``.
    """
    lamb = hasattr(ud, "LAMB_BDRY")
    s = (slice(1, -1), slice(1, -1))
    hplusx = mpv.wplus[0][s].T.reshape(-1)
    hplusy = mpv.wplus[1][s].T.reshape(-1)
    hcenter = mpv.wcenter[node.i1].T.reshape(-1)
    cor = tuple(c[s].reshape(-1) for c in coriolis)
    dinv = diag_inv[node.i1].T.reshape(-1)
    if lamb:            # lap2D_numba_test pads x periodically and y by mirroring, whatever bdry_type says
        return NodalHelmholtz2D(hplusx, hplusy, hcenter, cor, dinv, node.iicx, node.iicy, node.dx, node.dy,
                                False, False, device=device, y_mirror=True)
    return NodalHelmholtz2D(hplusx, hplusy, hcenter, cor, dinv, node.iicx, node.iicy, node.dx, node.dy,
                            _is_wall(ud.bdry_type[0]), _is_wall(ud.bdry_type[1]), device=device)


stencil_9pt = stencil_9pt_numba_test
