"""Seeded synthetic nanoparticles (the workloads' inputs).

All particles are cut from an fcc lattice with a site at the origin, then
displaced by seeded Gaussian noise; positions are float32 like the
reference's kernels use.  Random numbers come from numpy's PCG64
(``np.random.default_rng(seed)``).
"""
import numpy as np

__all__ = ['fcc_sites', 'fcc_sphere', 'fcc_nearest', 'displaced',
           'random_cube']

_FCC_BASIS = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])


def fcc_sites(a, radius):
    """All fcc sites (lattice constant a) within ``radius`` of the origin,
    ordered by distance then by coordinates."""
    m = int(np.ceil(radius / a)) + 1
    rng = np.arange(-m, m + 1)
    cells = np.stack(np.meshgrid(rng, rng, rng, indexing='ij'), -1).reshape(-1, 3)
    pts = (cells[:, None, :] + _FCC_BASIS[None]).reshape(-1, 3) * a
    d = np.sqrt((pts ** 2).sum(1))
    keep = d <= radius + 1e-9
    pts, d = pts[keep], d[keep]
    order = np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0], np.round(d, 9)))
    return pts[order]


def fcc_sphere(a, radius):
    """fcc sites with |x| <= radius (e.g. a=4.08, radius=10 gives 249 Au)."""
    return fcc_sites(a, radius)


def fcc_nearest(a, n):
    """The n fcc sites nearest the origin (ties broken by coordinates)."""
    # fcc number density is 4/a^3, so n sites fill a sphere of radius
    # a (3 n / (16 pi))^(1/3); start a little beyond it
    radius = a * (3.0 * n / (16.0 * np.pi)) ** (1.0 / 3.0) * 1.1 + a
    while True:
        pts = fcc_sites(a, radius)
        if len(pts) >= n:
            return pts[:n]
        radius *= 1.25


def displaced(sites, sigma, seed):
    """Sites plus N(0, sigma^2) displacements per coordinate, float32."""
    rng = np.random.default_rng(seed)
    return (sites + rng.normal(0.0, sigma, sites.shape)).astype(np.float32)


def random_cube(n, edge, seed):
    """n uniform random positions in a cube of the given edge, float32."""
    rng = np.random.default_rng(seed)
    return (rng.random((n, 3)) * edge).astype(np.float32)
