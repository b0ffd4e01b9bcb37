"""Ensembles of CDKLM16 members and the batched ensemble engine."""
