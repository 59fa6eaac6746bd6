"""Python plumbing around libsgx.so: a ctypes binding of the C ABI
(include/sgx.h), seeded workload generators and the sp5-lite table writer.

The compute path is the CUDA library; nothing in this package computes EOS or
PTE values itself.
"""
