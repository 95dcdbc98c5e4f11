/*
 * Force-included (g++ -include) when the reference kernel file
 * fdtd_calculations.cu is compiled as plain C++ for the CPU.  The kernels
 * become ordinary functions; the launch coordinates are thread-local globals
 * that ref_cpu.cpp sets before each call, and the __constant__ block becomes
 * plain globals that copySymbolsToDevice fills with memcpy.
 * Test infrastructure only: nothing here is part of the product.
 */
#pragma once
#include <cmath>
#include <math.h>  /* brings the float overload sqrt(float) into the global scope, as in device code */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cuda_runtime_api.h>
#undef __global__
#define __global__
#undef __constant__
#define __constant__
struct ref_cpu_idx3 { int x, y, z; };
static thread_local ref_cpu_idx3 threadIdx, blockIdx, blockDim;
#define cudaMemcpyToSymbol(sym, src, n) (memcpy(&(sym), (src), (n)), cudaSuccess)
#define cudaGetErrorString(e) "cuda error"
