// psf_ebe.cuh -- the matrix-free element-by-element operator on structured
// grids, shared by the solvers: one element matrix Ke0 (E = 1) scaled by the
// element modulus, gathered per node from the (up to) 4 / 8 surrounding
// elements of a zero-padded modulus array, so that no bounds branches are
// needed.  Node numbering follows the reference mesh generators
// (SquareMesh / CubeMesh): node (i, j[, k]) has id (ny+1) i + j
// (3D: ((ny+1) i + j)(nz+1) + k).
#pragma once

#include "psf_internal.cuh"

namespace psf {

template <class T>
struct KeT {
    T v[576];
};

struct Geo {
    int nx, ny, nz;
    long long nnodes;
};

__device__ __forceinline__ long long pad_index(const Geo &g, int ei, int ej, int ek, bool is3d) {
    return is3d ? ((long long)(ei + 1) * (g.ny + 2) + (ej + 1)) * (g.nz + 2) + (ek + 1)
                : (long long)(ei + 1) * (g.ny + 2) + (ej + 1);
}

// local node index of corner offset (di, dj, dk) (SquareMesh / ShapeFunction8Cubic order)
__device__ __forceinline__ int corner_local(int di, int dj, int dk) {
    return (di ? (dj ? 2 : 1) : (dj ? 3 : 0)) + 4 * dk;
}

// y[0..ndof) of node (i,j,k) = sum over surrounding elements; get(dof index) reads the input
template <class T, int KIND, class Get>
__device__ __forceinline__ void ebe_node(const Geo &g, const KeT<T> &Ke, const T *__restrict__ Ep, int i, int j,
                                         int k, Get get, T *y) {
    constexpr bool is3d = KIND == PSF_H8_SOLID;
    constexpr int ndof = KIND == PSF_Q4_PLANE_STRAIN ? 2 : (KIND == PSF_Q4_HEAT ? 1 : 3);
    constexpr int nen = is3d ? 8 : 4;
    constexpr int nk = nen * ndof;
#pragma unroll
    for (int a = 0; a < ndof; a++) y[a] = T(0);
#pragma unroll
    for (int ci = 0; ci < 2; ci++)
#pragma unroll
        for (int cj = 0; cj < 2; cj++)
#pragma unroll
            for (int ck = 0; ck < (is3d ? 2 : 1); ck++) {
                const int ei = i - 1 + ci, ej = j - 1 + cj, ek = is3d ? k - 1 + ck : 0;
                const T Ee = Ep[pad_index(g, ei, ej, ek, is3d)];
                const int li = corner_local(1 - ci, 1 - cj, is3d ? 1 - ck : 0);
                T ue[nk];
#pragma unroll
                for (int q = 0; q < nen; q++) {
                    const int qi = (q == 1 || q == 2 || q == 5 || q == 6), qj = (q == 2 || q == 3 || q == 6 || q == 7),
                              qk = q >= 4;
                    int ni = min(max(ei + qi, 0), g.nx), nj = min(max(ej + qj, 0), g.ny);
                    long long m;
                    if (is3d) {
                        int nkk = min(max(ek + qk, 0), g.nz);
                        m = ((long long)(g.ny + 1) * ni + nj) * (g.nz + 1) + nkk;
                    } else {
                        m = (long long)(g.ny + 1) * ni + nj;
                    }
#pragma unroll
                    for (int b = 0; b < ndof; b++) ue[q * ndof + b] = get(m * ndof + b);
                }
#pragma unroll
                for (int a = 0; a < ndof; a++) {
                    T acc = T(0);
                    const int row = (li * ndof + a) * nk;
#pragma unroll
                    for (int l = 0; l < nk; l++) acc += Ke.v[row + l] * ue[l];
                    y[a] += Ee * acc;
                }
            }
}

template <int KIND>
__device__ __forceinline__ void node_ijk(const Geo &g, long long n, int &i, int &j, int &k) {
    if (KIND == PSF_H8_SOLID) {
        k = (int)(n % (g.nz + 1));
        long long r = n / (g.nz + 1);
        j = (int)(r % (g.ny + 1));
        i = (int)(r / (g.ny + 1));
    } else {
        k = 0;
        j = (int)(n % (g.ny + 1));
        i = (int)(n / (g.ny + 1));
    }
}

template <int KIND>
__host__ __device__ constexpr int ndof_of() { return KIND == PSF_Q4_PLANE_STRAIN ? 2 : (KIND == PSF_Q4_HEAT ? 1 : 3); }

}  // namespace psf
