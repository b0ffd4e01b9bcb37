"""Global constants (counterpart of ``utils/config.py``)."""
soar_cutoff = 2
