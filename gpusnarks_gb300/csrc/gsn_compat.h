// Lets headers shared by host-only C++ and CUDA translation units use the
// CUDA function-space qualifiers.
#pragma once
#ifndef __CUDACC__
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
#endif
