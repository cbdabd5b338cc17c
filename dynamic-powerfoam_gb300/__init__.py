"""GB300-native bonded-DEM Newton solver (drop-in for the reference's
``bonded_dem_newton`` path).  Import as ``dpf_gb300``."""
from .foam import jittered_lattice_foam, gravity_load, regular_edges

__all__ = ['jittered_lattice_foam', 'gravity_load', 'regular_edges']
