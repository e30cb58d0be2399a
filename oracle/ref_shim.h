// ref_shim.h -- lets the reference's CUDA kernel sources compile as host C++ (TEST INFRASTRUCTURE).
//
// oracle/build_ref.sh force-includes this header when it compiles reference kernel sources with g++.
// Kernels become ordinary functions; a launch is emulated by setting the block/thread indices and calling
// the function once per thread, in order. This is exact for the kernels used here: none of them uses
// shared memory, barriers or atomics (the splats are run over one segment at a time, as the reference
// launches them).
#pragma once

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using std::fabs;
using std::floor;
using std::max;
using std::min;
using std::pow;
using std::sqrt;

struct dim3 {
    unsigned int x = 1, y = 1, z = 1;
    dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};

extern dim3 threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define IMUL(a, b) ((a) * (b))

typedef float cuflt;
typedef unsigned int uint;

// Runs kernel body `f` for every thread of the grid.
template <class F>
inline void ref_launch(dim3 grid, dim3 block, F f) {
    gridDim = grid;
    blockDim = block;
    for (unsigned bz = 0; bz < grid.z; ++bz)
        for (unsigned by = 0; by < grid.y; ++by)
            for (unsigned bx = 0; bx < grid.x; ++bx)
                for (unsigned tz = 0; tz < block.z; ++tz)
                    for (unsigned ty = 0; ty < block.y; ++ty)
                        for (unsigned tx = 0; tx < block.x; ++tx) {
                            blockIdx = dim3(bx, by, bz);
                            threadIdx = dim3(tx, ty, tz);
                            f();
                        }
}
