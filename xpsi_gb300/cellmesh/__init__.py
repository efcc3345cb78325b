"""Cell-mesh callables of the likelihood path (rays, integrator)."""
