"""Lagrangian drifter collections."""
