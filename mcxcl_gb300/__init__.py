"""mcxcl_gb300 -- the MCX-CL photon-transport path on GB300 (sm_103a).

Public API mirrors the reference's ``pmcxcl`` module: ``run``, ``gpuinfo``,
``version``; ``run_batch`` runs many simulations in one launch.  The C ABI is
in include/mcx_gb300.h.
"""
from .pmcxcl import MCXError, gpuinfo, keep_sessions, parse_config, run, run_batch, version  # noqa: F401

__version__ = "0.1.0"
__all__ = ["run", "run_batch", "keep_sessions", "gpuinfo", "version", "MCXError"]
