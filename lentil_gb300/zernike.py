"""Zernike OPD generators (host-side numpy, input preparation only).

Noll-ordered, Noll-normalised polynomials with lentil's coordinate
conventions (lentil/zernike.py:11-480)."""
from math import factorial

import numpy as np

from .util import centroid, mesh


def noll_to_nm(j):
    """Noll index -> (n, m) (lentil/zernike.py:348-391; Noll 1976 ordering:
    within a radial order, |m| increases, cosine terms take even j)."""
    if j < 1:
        raise ValueError('Noll index must be greater than zero')
    n = 0
    while (n + 1) * (n + 2) // 2 < j:
        n += 1
    first = n * (n + 1) // 2 + 1            # first Noll index of radial order n
    pos = j - first                          # 0-based position inside the order
    ms = [m for m in range(n % 2, n + 1, 2) for _ in ((0,) if m == 0 else (0, 1))]
    m = ms[pos]
    return n, (m if j % 2 == 0 else -m)


def radial(n, m, rho):
    """Zernike radial polynomial R_n^m (lentil/zernike.py:96-109)."""
    n, m = abs(int(n)), abs(int(m))
    if (n - m) % 2:
        return np.zeros_like(rho)
    out = np.zeros(np.shape(rho))
    for k in range((n - m) // 2 + 1):
        coef = (-1) ** k * factorial(n - k) / (
            factorial(k) * factorial((n + m) // 2 - k) * factorial((n - m) // 2 - k))
        out = out + coef * rho ** (n - 2 * k)
    return out


def zernike_coordinates(mask, shift=None, rotate=0):
    """(rho, theta) with rho = 1 at the farthest masked pixel from the
    mask centroid (lentil/zernike.py:444-480)."""
    mask = np.asarray(mask, dtype=bool)
    if shift is None:
        cen = centroid(mask)
        shift = (cen[0] - mask.shape[0] / 2, cen[1] - mask.shape[1] / 2)
    rr, cc = mesh(mask.shape, shift)
    r = np.hypot(rr, cc)
    rho = r / np.max(r * mask)
    a = (90 - rotate) * np.pi / 180
    theta = np.angle((-rr + 1j * cc) * np.exp(1j * a))
    return rho, theta


def zernike(mask, index, normalize=True, order='noll', rho=None, theta=None):
    """One Zernike polynomial over ``mask`` (lentil/zernike.py:11-93)."""
    if order != 'noll':
        raise ValueError('only Noll ordering is supported')
    mask = np.asarray(mask, dtype=bool)
    n, m = noll_to_nm(index)
    if rho is None:
        rho, theta = zernike_coordinates(mask)
    elif theta is None:
        raise ValueError('Both rho and theta must be specified')
    if m == 0:
        if n == 0:
            return mask.astype(float)
        z = radial(n, 0, rho) * (np.sqrt(n + 1) if normalize else 1.0)
    else:
        ang = np.cos(m * theta) if m > 0 else np.sin(m * theta)
        z = radial(n, m, rho) * ang * (np.sqrt(2 * (n + 1)) if normalize else 1.0)
    return z * mask


def zernike_compose(mask, coeffs, normalize=True, order='noll', rho=None, theta=None):
    """sum_j coeffs[j-1] Z_j over ``mask`` (lentil/zernike.py:112-180)."""
    mask = np.asarray(mask)
    if rho is None:
        rho, theta = zernike_coordinates(mask)
    out = np.zeros(mask.shape)
    for j, c in enumerate(np.asarray(coeffs).ravel(), start=1):
        out += c * zernike(mask, j, normalize, order, rho, theta)
    return out


def zernike_basis(mask, modes, vectorize=False, normalize=True, order='noll', rho=None,
                  theta=None):
    """Stack of Zernike polynomials (lentil/zernike.py:183-234)."""
    modes = np.atleast_1d(np.asarray(modes))
    mask = np.asarray(mask)
    if rho is None:
        rho, theta = zernike_coordinates(mask)
    basis = np.stack([zernike(mask, int(j), normalize, order, rho, theta) for j in modes])
    return basis.reshape(basis.shape[0], -1) if vectorize else basis
