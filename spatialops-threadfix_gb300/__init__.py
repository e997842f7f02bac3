"""GB300-native Nebo field-expression evaluation: Python host mirror of the C-ABI library.

The product is libnebo_gb300.so (CUDA kernels for sm_103a behind the C ABI declared in
include/nebo_gb300.h) plus the drop-in C++ headers under include/spatialops.  This package
loads the library with ctypes for the tests and the benchmark; it has no compute path of its
own and raises if the library is missing.
"""
