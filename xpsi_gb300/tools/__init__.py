"""Signal tools of the likelihood path (energy integration)."""
