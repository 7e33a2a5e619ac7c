"""kuramoto_gb300 -- Kuramoto network DP45 integrator for one GB300 (sm_103a).

Python mirror of the C ABI in ``include/kura.h`` (libkura.so).  The integration
itself runs in the persistent CUDA kernel of libkura; this module only moves
arguments.  There is no CPU fallback: importing works anywhere, but every
compute call needs the native library and a GPU and raises otherwise.
"""
from .native import (  # noqa: F401
    KuraError,
    MLP,
    MultiNetworks,
    Network,
    lib,
    lib_path,
    cli_path,
    random_inputs,
    volcano_factor,
    COUPLING_DENSE,
    COUPLING_VOLCANO,
    ENGINE_AUTO,
    ENGINE_PERSISTENT,
    ENGINE_TENSOR,
    ADJ_F32,
    ADJ_I8,
)

__all__ = ["KuraError", "MLP", "MultiNetworks", "Network", "lib", "lib_path", "cli_path", "random_inputs", "volcano_factor",
           "COUPLING_DENSE", "COUPLING_VOLCANO", "ENGINE_AUTO", "ENGINE_PERSISTENT", "ENGINE_TENSOR", "ADJ_F32", "ADJ_I8"]
