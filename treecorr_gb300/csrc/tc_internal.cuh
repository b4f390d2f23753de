// tc_internal.cuh -- shared types of the tree build, the traversal and the C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace tc {

enum { FLAT = 1, THREED = 2, SPHERE = 3 };
enum { EUCLIDEAN = 1, ARC = 4 };
enum { MIDDLE = 0, MEDIAN = 1, MEAN = 2, RANDOM = 3 };
enum { DN = 0, DK = 1, DG = 2 };   // payload: none, scalar, complex (Z, V, G, T, Q)

// Public data kinds (TC_NDATA.. in include/tcgpu.h: N, K, G, Z, V, T, Q = 0..6) as the
// payload kind and the spin of a complex value (include/ProjectHelper.h:63-71).
__host__ __device__ inline int kind_of(int d) { return d <= 1 ? d : DG; }
__host__ __device__ inline int spin_of(int d)
{
    return d == 2 ? 2 : d == 4 ? 1 : d == 5 ? 3 : d == 6 ? 4 : 0;
}

// Device status word: the first kernel error wins (atomicCAS from 0).
enum DevErr : int {
    DEV_OK = 0,
    DEV_STACK_OVERFLOW = 1,    // a traversal warp stack would overflow
    DEV_SPILL_OVERFLOW = 2,    // spill buffer too small
    DEV_DEGENERATE_SPLIT = 3,  // mean split failed on a large cell whose points differ
    DEV_BAD_CHILD = 4,         // traversal asked to split a leaf (inconsistent tree)
    DEV_TASK_OVERFLOW = 5,     // build task list overflow
    DEV_COPY_TIMEOUT = 6,      // an asynchronous copy into shared memory did not complete
};

// Catalog points during the build (structure of arrays, one of two ping-pong buffers).
struct Points {
    double* x;
    double* y;
    double* z;
    double* wp;   // position weight
    float* w;     // weight, float like include/Cell.h:93
    float* d1;    // w*k (K) or Re(w*g) (G), float like include/Cell.h:154,190
    float* d2;    // Im(w*g)
    int* idx;     // original index
};

// Cell arrays, indexed by cell id.  Internal cell that splits [s,e) at m: id m-1.
// Leaf (single point or list leaf) starting at point s: id (n-1)+s.  2n-1 ids in total.
struct Cells {
    double* x;
    double* y;
    double* z;
    float* size;
    float* w;
    float* d1;
    float* d2;
    int* n;
    int* start;
    int* left;    // -1 for a leaf
    int* right;
    int* parent;  // -1 for a top-level cell's root
};

// Traversal record of one cell, 64 bytes, read with four 16-byte loads.
//   a = (x_hi, y_hi, z_hi, size)   b = (x_lo, y_lo, z_lo, w)
//   c = (d1, d2, n (int bits), left id (int bits))   d = (right id (int bits), pad...)
// x_hi = float(x), x_lo = float(x - x_hi): differences of nearby cells keep ~48 bits.
struct __align__(16) TCell {
    float4 a, b, c, d;
};

// Work item of the build: a cell to process, with its place in the tree.
struct BuildTask {
    int s, e;          // point range
    int parent;        // parent cell id (-1 for the root)
    int side;          // 0 = left child, 1 = right child
    int mintop, maxtop;// remaining top-level recursion counters (SetupTopLevelCells)
    int intop;         // 1 while still in the top-level phase
    int buf;           // which point buffer holds [s,e)
};

struct BuildParams {
    int coords, dkind, split, brute;
    int spin;          // complex payloads: the spin of the parallel transport
    double minsizesq, maxsizesq;
    int n;
};


static constexpr int CH = 4096;        // points per chunk in the cooperative levels
static constexpr int CB = 256;         // threads per chunk block
static constexpr int SMALL = 2048;     // cells at most this big are finished by one warp

struct Part1 {   // chunk partial of pass 1
    double sx, sy, sz, swp, sw;
    double xmin, xmax, ymin, ymax, zmin, zmax;
};
struct Part2 {   // chunk partial of pass 2
    double sizesq, pr, pi;
    int nleft, pad;
};
struct TaskStats {  // per cooperative task, filled by combine1 / combine2
    double cx, cy, cz;
    double splitval;
    int axis;
    float w;
    int mid;        // split point, or -1 for a leaf
    int copy;       // 1 if the leaf's points must be copied to buffer 0
    int allsame;    // 1 if every point shares the split coordinate
    int byindex;    // 1 if the split is by position (median fallback)
};
struct Chunk {
    int task, cs, ce;
    int leftoff, rightoff;   // filled by combine2
};

struct WTask { int s, e, parent, meta; };   // meta: side | intop<<1 | buf<<2 | mintop<<8 | maxtop<<20

// Device scratch of the build, grown on demand and kept by the field.
struct BuildScratch {
    BuildTask* tasks = nullptr;     // cooperative tasks of the current level
    int* chunk0 = nullptr;          // first chunk of each task (+1 sentinel)
    Chunk* chunks = nullptr;
    Part1* part1 = nullptr;
    Part2* part2 = nullptr;
    TaskStats* stats = nullptr;
    BuildTask* big_next = nullptr;  // cooperative tasks of the next level
    BuildTask* small = nullptr;     // warp tasks (capacity n)
    int* counters = nullptr;        // [0] next cooperative count, [1] warp task count
    WTask* wstack = nullptr;        // per-warp-task stacks (capacity n)
    int cap_tasks = 0, cap_chunks = 0;
};


// Great-circle angle from the squared chord of two unit vectors, theta = 2 asin(c/2), in
// FP32.  For c < 0.25 the Maclaurin series of arcsin to x^7 (x = c/2 <= 0.125; the first
// omitted term, 35 x^9 / 1152, is below 2e-9 of x) replaces the library call.
__device__ __forceinline__ float arc_from_chord_sq(float dsq)
{
    const float c = sqrtf(dsq);
    if (c < 0.25f) {
        const float x = 0.5f * c, x2 = x * x;
        return 2.f * x * (1.f + x2 * (1.f / 6.f + x2 * (3.f / 40.f + x2 * (5.f / 112.f))));
    }
    return 2.f * asinf(0.5f * c);
}

}  // namespace tc
