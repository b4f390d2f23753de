// kmeans.hpp -- k-means patch finding on a field's tree (kmeans.cu): the reference's
// KMeansInit{Tree,Rand,KMPP}, KMeansRun, KMeansAssign (src/KMeans.cpp:743-849) and the
// catalog-level QuickAssign / SelectPatch (src/KMeans.cpp:890-1011).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tc_internal.cuh"

namespace tc {

// What the k-means code needs of a built field.
struct KMField {
    int coords = 0;
    int64_t n = 0;           // points
    int ncap = 0;            // cell ids (2n - 1)
    Cells cells = {};
    const int* d_tops = nullptr;   // top-level cell ids, in the reference's getCells() order
    int ntop = 0;
    const int* idx = nullptr;      // original index of each sorted point
    double size = 0.;              // BaseField::getSize(): sqrt of the overall size^2
};

// centers: npatch rows of 2 (Flat) or 3 (ThreeD, Sphere) doubles, host memory.
// Reseeds the k-means initialisations' urand stream for a non-zero seed (the field
// constructor's seed, src/Field.cpp:160).
void km_seed(long long seed);
int kmeans_init_tree(const KMField& F, double* centers, int npatch, long long seed,
                     cudaStream_t st);
int kmeans_init_rand(const KMField& F, double* centers, int npatch, long long seed,
                     cudaStream_t st);
int kmeans_init_kmpp(const KMField& F, double* centers, int npatch, long long seed,
                     cudaStream_t st);
// iters_out (nullable): iterations run.
int kmeans_run(const KMField& F, double* centers, int npatch, int max_iter, double tol,
               bool alt, cudaStream_t st, int* iters_out);
// patches: n entries (host), the patch of each point in its original order.
int kmeans_assign(const KMField& F, const double* centers, int npatch, int64_t* patches,
                  cudaStream_t st);
// Nearest centre of every point (QuickAssign) / whether patch is the nearest (SelectPatch).
// z == nullptr selects the 2-d form.  on_device: x, y, z and out are device pointers.
int quick_assign(const double* centers, int npatch, const double* x, const double* y,
                 const double* z, int64_t n, int64_t* out, bool on_device, cudaStream_t st);
int select_patch(int patch, const double* centers, int npatch, const double* x,
                 const double* y, const double* z, int64_t n, int64_t* use, bool on_device,
                 cudaStream_t st);

}  // namespace tc
