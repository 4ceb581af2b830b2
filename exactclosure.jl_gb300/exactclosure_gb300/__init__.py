"""GB300 (sm_103a) implementation of the DNS-aided LES hot path of
agdestein/ExactClosure.jl behind the libexc C ABI (include/exc.h).

``navierstokes`` mirrors the reference's ``NavierStokes`` module
(``src/N.jl``) on top of the ABI.
"""
from . import _lib
from ._lib import EXC_F32, EXC_F64, ExcError, lib

__all__ = ["EXC_F32", "EXC_F64", "ExcError", "lib", "_lib"]
