"""Likelihood extension of the path (background marginalisation)."""
