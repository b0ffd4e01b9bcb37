"""Shallow-water simulators (CDKLM16) and the stochastic model error."""
