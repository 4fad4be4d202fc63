/*
 * ref_shim.h -- force-included when the checker recipe in oracle/Makefile
 * compiles the reference's own sources.  TEST INFRASTRUCTURE ONLY.
 *
 * The reference includes two NVIDIA CUDA-samples headers (helper_cuda.h,
 * helper_string.h) that do not compile under CUDA 13; the recipe defines
 * their include guards so their bodies are skipped, and this file supplies
 * the one macro the reference uses from them (checkCudaErrors).  For the
 * host-only g++ build of fault.cpp it also stubs the two CUDA names that
 * functions.h declares unconditionally (__global__, cublasHandle_t).
 */
#ifndef QDEQ_REF_SHIM_H
#define QDEQ_REF_SHIM_H
#include <stdio.h>
#include <stdlib.h>
#if defined(GPU)
#include <cuda_runtime.h>
#include <cublas_v2.h>
#define checkCudaErrors(x)                                                   \
    do {                                                                     \
        int e__ = (int)(x);                                                  \
        if (e__ != 0) {                                                      \
            fprintf(stderr, "CUDA error %d at %s:%d\n", e__, __FILE__, __LINE__); \
            exit(1);                                                         \
        }                                                                    \
    } while (0)
#else
#define __global__
#define __constant__
typedef void *cublasHandle_t;
#endif
#endif
