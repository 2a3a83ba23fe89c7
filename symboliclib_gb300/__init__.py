"""symboliclib_gb300: GB300 execution engine for SymbolicLib ComputeUnit plans.

The product is native code: the C++ front end and CUDA engine in
``lib/libsymgb.so`` (C ABI in ``include/symgb.h``, C++ API in
``include/symgb/ComputeUnit.hpp``).  This package builds it in-tree
(:mod:`symboliclib_gb300.build`) and binds it for Python callers
(:mod:`symboliclib_gb300.native`)."""
