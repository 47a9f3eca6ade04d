"""Rayleigh-Benard solvers (navier/ of pypde)."""
