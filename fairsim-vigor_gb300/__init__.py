"""fairsim-vigor_gb300: GB300-native (sm_103a) 2D SIM reconstruction behind fairSIM's API.

Layout:
  csrc/          CUDA kernels and the C ABI (include/fairsim_gb300.h), built by build.py
  native.py      ctypes binding of lib/libfairsim_gb300.so
  vectors.py     Vector API (AccelVectorFactory / Vec2d.Real / Vec2d.Cplx) on device memory
  algorithm.py   SimAlgorithm / BandSeparation / SimUtils / Correlation / WienerFilter / OTF writers
  plan.py        fused batched reconstruction plans, CUDA-graph batches, host-buffer batches
                 and the served (live) form
  replicas.py    multi-GPU form: disjoint dataset shares per rank, max-over-ranks timing
  ingest.py      live stream ingest: LIVESIM frame headers, SIM sequence detection
  sim_param.py   SimParam / SimParam.Dir / OtfProvider records
  conf.py        fairSIM / VIGOR XML configuration files (utils/Conf), live channel settings
  synth.py       seeded synthetic SIM datasets
"""
from .sim_param import Dir, OtfProvider, SimParam  # noqa: F401
from . import synth  # noqa: F401
from . import conf  # noqa: F401
from . import native  # noqa: F401


def __getattr__(name):
    # vector/algorithm modules load the native library lazily
    import importlib

    if name in ("vectors", "algorithm", "plan", "replicas", "autotune", "ingest"):
        return importlib.import_module("." + name, __name__)
    if name in ("AccelVectorFactory", "Vec2dReal", "Vec2dCplx"):
        return getattr(importlib.import_module(".vectors", __name__), name)
    if name in ("SimAlgorithm", "BandSeparation", "SimUtils", "Correlation", "WienerFilter", "OtfVectors",
                "RLDeconvolution"):
        return getattr(importlib.import_module(".algorithm", __name__), name)
    raise AttributeError(name)
