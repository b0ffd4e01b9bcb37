"""GB300-native (sm_103a) CDKLM16 ocean model engine with GPU Ocean's Python API.

Sub-packages mirror the reference's layout so that code written against
``gpuocean`` can switch imports:

* ``gpuocean_gb300.SWEsimulators``  CDKLM16, OceanStateNoise
* ``gpuocean_gb300.drifters``       GPU/CPU drifter collections
* ``gpuocean_gb300.ensembles``      ensembles and the batched ensemble engine
* ``gpuocean_gb300.utils``          Common (device arrays, BCs, bathymetry), forcing

All numerical work runs in ``libgpuocean_gb300.so`` (built from ``csrc/``).
"""
__version__ = "0.1.0"
