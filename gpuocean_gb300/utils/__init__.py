"""Device runtime, boundary conditions, bathymetry and forcing."""
