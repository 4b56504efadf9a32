// Name -> kernel table for the reference's GPU kernels compiled ahead of
// time (test infrastructure, never shipped).  The reference launches its
// kernels by name through an NVRTC-built module that it loads and unloads
// around every launch (src/cudaUtils.cpp:197-218); the oracle's harness
// compiles the same kernel sources with nvcc instead and launches them by
// the same names through this table (gpu_shim.cpp).
#pragma once
#include <map>
#include <string>

std::map<std::string, const void *> &ref_kernel_table();

struct RefKernelReg {
  RefKernelReg(const char *name, const void *fn) { ref_kernel_table()[name] = fn; }
};

#define REF_KERNEL(k) static RefKernelReg ref_reg_##k(#k, (const void *)(k));
