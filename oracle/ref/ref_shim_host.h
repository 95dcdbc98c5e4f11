/*
 * Force-included (nvcc -include) when the reference host file fdtd.cu is
 * compiled into the reference harness library.  The system headers are
 * included first so that they see the real platform; afterwards __APPLE__ is
 * defined, which makes the reference compile out the body of
 * setupMurBoundary (its own #ifndef __APPLE__, fdtd.cu:944) -- the only part
 * of the file written with C99 complex types, which C++ compilers reject.
 * The Mur slabs therefore come from the oracle's C99 restatement.
 * Test infrastructure only.
 */
#pragma once
#include <stdlib.h>
#include <stdio.h>
#include <math.h>
#include <complex.h>
#include <unistd.h>
#include <pthread.h>
#include <cuda_runtime_api.h>
#define __APPLE__ 1
