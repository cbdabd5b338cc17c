"""Synthetic jittered-lattice power foams (the solver's input format).

A foam is the set of arguments of ``NewtonBonds(points, radii, pairs, areas,
masses, fixed, contacts=None, young, shear)``.  Bonds are the edges of the
regular (weighted Delaunay) triangulation of the sites, taken from the lower
hull of the lifted points ``(x, |x|^2 - w)`` exactly as the reference builds
its bond candidates (``experiments/powersim_bread_demo.py:114-133``,
``benchmark.py:25-53``).

Generator choices (not fixed by the reference):

* sites are ``(g + 1/2) h + U[-0.2, 0.2] h`` on an ``m^3`` lattice of spacing
  ``h = 1/m`` (box aspect ratios stretch the unit cube), listed in Morton order
  of their lattice cell so that bonded sites sit close in memory;
* power weights are ``U[0, 0.01] * (8 h)^2``: literal ``U[0, 0.01]`` weights
  exceed ``h^2`` for ``m >= 16`` and hide whole sites (1,055 of 4,096 at
  ``m = 16``); scaling by ``(8h)^2`` keeps the ``m = 8`` weights literal and
  hides none, giving about 7.4 bonds per site;
* bond cross-section areas are ``U[0.5, 1] h^2``; rest lengths are the
  initial distances; contacts are the classical ball contacts;
* radii (lever arms and rotational inertia) are ``h/2``;
* ``young = E`` and ``shear = E / (2 (1 + nu))``;
* sites with ``z < 0.05`` (in unit-cube coordinates) are fixed.
"""
import numpy as np
from scipy.spatial import ConvexHull


def morton_order(m):
    """Lattice indices (m^3, 3) sorted by 3-D Morton code."""
    g = np.stack(np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing='ij'), -1).reshape(-1, 3)
    code = np.zeros(len(g), dtype=np.int64)
    for bit in range(int(np.ceil(np.log2(max(m, 2))))):
        for axis in range(3):
            code |= ((g[:, axis] >> bit) & 1).astype(np.int64) << (3*bit + axis)
    return g[np.argsort(code, kind='stable')]


def regular_edges(points, weights):
    """Edges of the regular triangulation from the lower lifted convex hull.

    Follows ``experiments/powersim_bread_demo.py:120-133``: centre and scale the
    points, lift to ``|z|^2 - w/scale^2``, keep facets whose outward normal has a
    negative lift component, and collect the unique sorted simplex edges.
    """
    p = np.asarray(points, dtype=np.float64)
    scale = np.ptp(p, axis=0).max()
    z = (p - p.mean(0))/scale
    lifted = np.column_stack((z, (z*z).sum(1) - np.asarray(weights)/scale**2))
    hull = ConvexHull(lifted)
    lower = hull.simplices[hull.equations[:, -2] < -1e-10]
    pairs = np.concatenate([lower[:, [a, b]] for a in range(4) for b in range(a+1, 4)])
    return np.unique(np.sort(pairs, axis=1), axis=0).astype(np.int64)


def jittered_lattice_foam(m, seed=0, *, aspect=(1., 1., 1.), young=1e5, poisson=.3,
                          density=1000., fixed_below=.05, mass=None):
    """Build a jittered ``m^3`` lattice foam; returns a dict of solver inputs.

    ``mass`` overrides the per-site mass (default ``density * h^3 * prod(aspect)``).
    The dict also carries ``h`` and ``unit`` (site coordinates in the unit cube)
    for boundary conditions and loads.
    """
    rng = np.random.default_rng(seed)
    h = 1./m
    lattice = morton_order(m)
    unit = (lattice + .5)*h + rng.uniform(-.2, .2, lattice.shape)*h
    weights = rng.uniform(0., .01, len(unit))*(8*h)**2
    aspect = np.asarray(aspect, dtype=np.float64)
    points = unit*aspect
    pairs = regular_edges(points, weights*float(np.prod(aspect))**(2/3))
    areas = rng.uniform(.5, 1., len(pairs))*h*h
    cell = density*h**3*float(np.prod(aspect))
    masses = np.full(len(points), cell if mass is None else mass)
    return dict(points=points, radii=np.full(len(points), .5*h), pairs=pairs, areas=areas,
                masses=masses, fixed=unit[:, 2] < fixed_below, contacts=None,
                young=float(young), shear=float(young)/(2*(1+poisson)), h=h, unit=unit)


def gravity_load(foam, g=9.81):
    """External (N, 6) load: weight ``-m g`` on z, zero on fixed sites and torques."""
    load = np.zeros((len(foam['points']), 6))
    load[:, 2] = -g*np.asarray(foam['masses'])
    load[np.asarray(foam['fixed'])] = 0.
    return load
