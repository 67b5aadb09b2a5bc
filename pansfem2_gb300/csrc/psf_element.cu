// psf_element.cu -- element stiffness / conductivity matrices on the device.
//
// Compiled with --fmad=false: every product and sum is rounded on its own, in
// the order of the reference element routines, so the matrix equals the
// reference's PlaneStrainStiffness / HeatTransfer / SolidLinearIsotropicElastic
// output bit for bit.  Structured grids share one geometry, so one matrix per
// context (element 0, E = 1) serves every element, scaled by E_e.
#include "psf_internal.cuh"

namespace psf {
namespace {

// C = A(r x k) B(k x c), sums from 0 in k order (Matrix::operator*, Matrix.h:243-256)
__device__ void mm(const double *A, const double *B, double *C, int r, int k, int c) {
    for (int i = 0; i < r; i++)
        for (int j = 0; j < c; j++) {
            double v = 0.0;
            for (int q = 0; q < k; q++) v += A[i * k + q] * B[q * c + j];
            C[i * c + j] = v;
        }
}

// sum over q of a[q] * b[q * bstride] for the q where row i of A and column j of B can both be
// nonzero, in q order, starting from the first such product (0.0 when there is none)
template <int K, class MA, class MB>
__device__ __forceinline__ double dot_s(const double *a, const double *b, int bstride, int i, int j) {
    double v = 0.0;
    bool any = false;
#pragma unroll
    for (int q = 0; q < K; q++)
        if (MA::nz(i, q) && MB::nz(q, j)) {
            const double p = a[q] * b[q * bstride];
            v = any ? v + p : p;
            any = true;
        }
    return v;
}

// The same product with the structural zeros of A and B left out, and the leading 0.0 +.
// MA::nz(i, q) and MB::nz(q, j) say where A and B can be nonzero; after unrolling they are
// constants, so the skipped terms cost nothing.  For finite factors the result differs from
// the reference's sum at most in the sign of a zero: a skipped term is +-0, and adding +-0
// leaves a nonzero sum as it is.  Every such value ends in a product and then in a sum that
// starts from +0.0 (the element matrix), and a sum that starts from +0 is never -0 (x + (-x)
// rounds to +0), so the element matrix is the reference's bit for bit.
template <int R, int K, int C, class MA, class MB>
__device__ __forceinline__ void mm_s(const double *A, const double *B, double *Out) {
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < C; j++) Out[i * C + j] = dot_s<K, MA, MB>(A + i * K, B + j, C, i, j);
}
// plane strain, Q4: B (3 x 8) rows exx, eyy, gxy over (ux0, uy0, ux1, ...); D (3 x 3)
struct NzB2 { static __device__ constexpr bool nz(int r, int c) { return r == 2 || (c & 1) == r; } };
struct NzBt2 { static __device__ constexpr bool nz(int r, int c) { return NzB2::nz(c, r); } };
struct NzD2 { static __device__ constexpr bool nz(int r, int c) { return (r < 2 && c < 2) || (r == 2 && c == 2); } };
struct NzBtD2 {
    static __device__ constexpr bool nz(int r, int c) {
        return (NzBt2::nz(r, 0) && NzD2::nz(0, c)) || (NzBt2::nz(r, 1) && NzD2::nz(1, c)) ||
               (NzBt2::nz(r, 2) && NzD2::nz(2, c));
    }
};
// solid, H8: B (6 x 24) rows exx, eyy, ezz, gxy, gyz, gzx over (ux0, uy0, uz0, ...); C (6 x 6)
struct NzB3 {
    static __device__ constexpr bool nz(int r, int c) {
        return r < 3 ? c % 3 == r : (r == 3 ? c % 3 != 2 : (r == 4 ? c % 3 != 0 : c % 3 != 1));
    }
};
struct NzBt3 { static __device__ constexpr bool nz(int r, int c) { return NzB3::nz(c, r); } };
struct NzC3 { static __device__ constexpr bool nz(int r, int c) { return (r < 3 && c < 3) || r == c; } };
struct NzBtC3 {
    static __device__ constexpr bool nz(int r, int c) {
        return (NzBt3::nz(r, 0) && NzC3::nz(0, c)) || (NzBt3::nz(r, 1) && NzC3::nz(1, c)) ||
               (NzBt3::nz(r, 2) && NzC3::nz(2, c)) || (NzBt3::nz(r, 3) && NzC3::nz(3, c)) ||
               (NzBt3::nz(r, 4) && NzC3::nz(4, c)) || (NzBt3::nz(r, 5) && NzC3::nz(5, c));
    }
};

__device__ double det2(const double *v) { return v[0] * v[3] - v[1] * v[2]; }
// Matrix::Determinant 3x3 term order (Matrix.h:333-334)
__device__ double det3(const double *v) {
    return -v[8] * v[1] * v[3] - v[7] * v[5] * v[0] - v[2] * v[4] * v[6] + v[6] * v[1] * v[5] +
           v[7] * v[3] * v[2] + v[0] * v[4] * v[8];
}
// Matrix::Inverse (Matrix.h:346-360): signed cofactor determinants of the
// transposed position, then each entry divided by the determinant
__device__ void inv_n(const double *A, int n, double *inv) {
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            // cofactor of (row j, column i)
            double cof[4];
            int m = 0;
            for (int a = 0; a < n; a++) {
                if (a == j) continue;
                for (int b = 0; b < n; b++) {
                    if (b == i) continue;
                    cof[m++] = A[a * n + b];
                }
            }
            double d = (n == 2) ? cof[0] : det2(cof);
            inv[i * n + j] = (((i + j) & 1) ? -1.0 : 1.0) * d;
        }
    double det = (n == 2) ? det2(A) : det3(A);
    for (int k = 0; k < n * n; k++) inv[k] /= det;
}

__device__ void gauss_q4(int g, double *r) {
    const double a = 1.0 / sqrt(3.0);
    r[0] = (g == 0 || g == 2) ? -a : a;   // (-,-), (+,-), (-,+), (+,+)
    r[1] = (g < 2) ? -a : a;
}
__device__ void gauss_h8(int g, double *r) {
    const double a = 1.0 / sqrt(3.0);
    const int sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
              sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    r[0] = sx[g] < 0 ? -a : a;
    r[1] = sy[g] < 0 ? -a : a;
    r[2] = sz[g] < 0 ? -a : a;
}
__device__ void dndr_q4(const double *r, double *d) {
    d[0] = -0.25 * (1.0 - r[1]); d[1] = 0.25 * (1.0 - r[1]);
    d[2] = 0.25 * (1.0 + r[1]);  d[3] = -0.25 * (1.0 + r[1]);
    d[4] = -0.25 * (1.0 - r[0]); d[5] = -0.25 * (1.0 + r[0]);
    d[6] = 0.25 * (1.0 + r[0]);  d[7] = 0.25 * (1.0 - r[0]);
}
__device__ void dndr_h8(const double *r, double *d) {
    const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
                 sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    // ShapeFunction8Cubic::dNdr (ShapeFunction.h:318-329): +-0.125 times the two
    // other factors, in the order the reference writes them
    for (int n = 0; n < 8; n++) {
        double c = (sx[n] < 0 ? -0.125 : 0.125);
        d[n] = c * (sy[n] < 0 ? 1.0 - r[1] : 1.0 + r[1]) * (sz[n] < 0 ? 1.0 - r[2] : 1.0 + r[2]);
        c = (sy[n] < 0 ? -0.125 : 0.125);
        d[8 + n] = c * (sz[n] < 0 ? 1.0 - r[2] : 1.0 + r[2]) * (sx[n] < 0 ? 1.0 - r[0] : 1.0 + r[0]);
        c = (sz[n] < 0 ? -0.125 : 0.125);
        d[16 + n] = c * (sx[n] < 0 ? 1.0 - r[0] : 1.0 + r[0]) * (sy[n] < 0 ? 1.0 - r[1] : 1.0 + r[1]);
    }
}

// PlaneStrainStiffness (PlaneStrain.h:20-58): Ke = sum_g B^T D B J t w0 w1, accumulated in
// registers and stored once.  The products skip the structural zeros of B and D (mm_s) and
// the weights (both 1.0: x * 1.0 is x), which leaves every entry as the reference's
__device__ void ke_planestrain(const double *X, double E, double V, double t, double *Ke_out) {
    double D[9] = {1.0 - V, V, 0.0, V, 1.0 - V, 0.0, 0.0, 0.0, 0.5 * (1.0 - 2.0 * V)};
    const double sc = E / ((1.0 - 2.0 * V) * (1.0 + V));
#pragma unroll
    for (int k = 0; k < 9; k++) D[k] *= sc;
    double Ke[64];
#pragma unroll
    for (int k = 0; k < 64; k++) Ke[k] = 0.0;
#pragma unroll 1
    for (int g = 0; g < 4; g++) {
        double r[2], dN[8], J2[4], iv[4], dX[8], B[24], Bt[24], BtD[24];
        gauss_q4(g, r);
        dndr_q4(r, dN);
        mm(dN, X, J2, 2, 4, 2);
        const double J = det2(J2);
        inv_n(J2, 2, iv);
        mm(iv, dN, dX, 2, 2, 4);
#pragma unroll
        for (int n = 0; n < 4; n++) {
            B[2 * n] = dX[n];          B[2 * n + 1] = 0.0;
            B[8 + 2 * n] = 0.0;        B[8 + 2 * n + 1] = dX[4 + n];
            B[16 + 2 * n] = dX[4 + n]; B[16 + 2 * n + 1] = dX[n];
        }
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 3; j++) Bt[i * 3 + j] = B[j * 8 + i];
        mm_s<8, 3, 3, NzBt2, NzD2>(Bt, D, BtD);
#pragma unroll
        for (int i = 0; i < 8; i++)   // (B^T D) B entry by entry, each added to Ke at once
#pragma unroll
            for (int j = 0; j < 8; j++) Ke[i * 8 + j] += dot_s<3, NzBtD2, NzB2>(BtD + i * 3, B + j, 8, i, j) * J * t;
    }
#pragma unroll
    for (int k = 0; k < 64; k += 2) *reinterpret_cast<double2 *>(Ke_out + k) = make_double2(Ke[k], Ke[k + 1]);
}

// PlaneStrainStiffness<ShapeFunction3Triangle, Gauss1Triangle> (PlaneStrain.h:20-58 with
// ShapeFunction.h:87-117 and GaussIntegration.h:64-81): one point (1/3, 1/3), weights 1/sqrt(2)
__device__ void ke_planestrain_t3(const double *X, double E, double V, double t, double *Ke) {
    double D[9] = {1.0 - V, V, 0.0, V, 1.0 - V, 0.0, 0.0, 0.0, 0.5 * (1.0 - 2.0 * V)};
    const double sc = E / ((1.0 - 2.0 * V) * (1.0 + V));
    for (int k = 0; k < 9; k++) D[k] *= sc;
    const double dN[6] = {1.0, 0.0, -1.0, 0.0, 1.0, -1.0};   // dN/dr, constant
    const double w = 1.0 / sqrt(2.0);
    double J2[4], iv[4], dX[6], B[18], Bt[18], BtD[18], K[36];
    mm(dN, X, J2, 2, 3, 2);
    const double J = det2(J2);
    inv_n(J2, 2, iv);
    mm(iv, dN, dX, 2, 2, 3);
    for (int n = 0; n < 3; n++) {
        B[2 * n] = dX[n];          B[2 * n + 1] = 0.0;
        B[6 + 2 * n] = 0.0;        B[6 + 2 * n + 1] = dX[3 + n];
        B[12 + 2 * n] = dX[3 + n]; B[12 + 2 * n + 1] = dX[n];
    }
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 3; j++) Bt[i * 3 + j] = B[j * 6 + i];
    mm(Bt, D, BtD, 6, 3, 3);
    mm(BtD, B, K, 6, 3, 6);
    for (int k = 0; k < 36; k++) Ke[k] = 0.0 + K[k] * J * t * w * w;
}

// HeatTransfer (HeatTransfer.h:19-43)
__device__ void ke_heat(const double *X, double alpha, double t, double *Ke) {
    for (int k = 0; k < 16; k++) Ke[k] = 0.0;
    for (int g = 0; g < 4; g++) {
        double r[2], dN[8], J2[4], iv[4], B[8], Bt[8], K[16];
        gauss_q4(g, r);
        dndr_q4(r, dN);
        mm(dN, X, J2, 2, 4, 2);
        const double J = det2(J2);
        inv_n(J2, 2, iv);
        mm(iv, dN, B, 2, 2, 4);
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 2; j++) Bt[i * 2 + j] = B[j * 4 + i];
        mm(Bt, B, K, 4, 2, 4);
        for (int k = 0; k < 16; k++) Ke[k] += K[k] * J * alpha * t * 1.0 * 1.0;
    }
}

// SolidLinearIsotropicElastic (Solid.h:20-64)
__device__ void ke_solid(const double *X, double E, double V, double *Ke, double *wk) {
    double C[36];
    for (int k = 0; k < 36; k++) C[k] = 0.0;
    C[0] = 1.0 - V; C[1] = V;  C[2] = V;
    C[6] = V;  C[7] = 1.0 - V; C[8] = V;
    C[12] = V; C[13] = V;      C[14] = 1.0 - V;
    C[21] = 0.5 * (1.0 - 2.0 * V);
    C[28] = 0.5 * (1.0 - 2.0 * V);
    C[35] = 0.5 * (1.0 - 2.0 * V);
    const double sc = E / ((1.0 + V) * (1.0 - 2.0 * V));
    for (int k = 0; k < 36; k++) C[k] *= sc;
    for (int k = 0; k < 576; k++) Ke[k] = 0.0;
    double *B = wk, *Bt = wk + 144, *BtC = wk + 288, *K = wk + 432;
    for (int g = 0; g < 8; g++) {
        double r[3], dN[24], J3[9], iv[9], dX[24];
        gauss_h8(g, r);
        dndr_h8(r, dN);
        mm(dN, X, J3, 3, 8, 3);
        const double J = det3(J3);
        inv_n(J3, 3, iv);
        mm(iv, dN, dX, 3, 3, 8);
        for (int k = 0; k < 144; k++) B[k] = 0.0;
        for (int n = 0; n < 8; n++) {
            const double d0 = dX[n], d1 = dX[8 + n], d2 = dX[16 + n];
            B[3 * n] = d0;
            B[24 + 3 * n + 1] = d1;
            B[48 + 3 * n + 2] = d2;
            B[72 + 3 * n] = d1;      B[72 + 3 * n + 1] = d0;
            B[96 + 3 * n + 1] = d2;  B[96 + 3 * n + 2] = d1;
            B[120 + 3 * n] = d2;     B[120 + 3 * n + 2] = d0;
        }
        for (int i = 0; i < 24; i++)
            for (int j = 0; j < 6; j++) Bt[i * 6 + j] = B[j * 24 + i];
        mm_s<24, 6, 6, NzBt3, NzC3>(Bt, C, BtC);        // structural zeros skipped, as in ke_planestrain
        mm_s<24, 6, 24, NzBtC3, NzB3>(BtC, B, K);
        for (int k = 0; k < 576; k++) Ke[k] += K[k] * J;   // the three weights are 1.0
    }
}

// one thread: the element matrix of element 0 with its actual node coordinates
__global__ void ke_element0_kernel(int kind, int nx, int ny, int nz, double lx, double ly, double lz,
                                   double E, double V, double t, double *Ke, double *wk) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    // SquareMesh coordinates x*(i/(T)nx) of element 0's nodes, in the element's node order
    double X[24];
    if (kind == PSF_H8_SOLID) {
        const int ci[8] = {0, 1, 1, 0, 0, 1, 1, 0}, cj[8] = {0, 0, 1, 1, 0, 0, 1, 1},
                  ck[8] = {0, 0, 0, 0, 1, 1, 1, 1};
        for (int n = 0; n < 8; n++) {
            X[3 * n + 0] = lx * (ci[n] / (double)nx);
            X[3 * n + 1] = ly * (cj[n] / (double)ny);
            X[3 * n + 2] = lz * (ck[n] / (double)nz);
        }
        ke_solid(X, E, V, Ke, wk);
    } else {
        const int ci[4] = {0, 1, 1, 0}, cj[4] = {0, 0, 1, 1};
        for (int n = 0; n < 4; n++) {
            X[2 * n + 0] = lx * (ci[n] / (double)nx);
            X[2 * n + 1] = ly * (cj[n] / (double)ny);
        }
        if (kind == PSF_Q4_PLANE_STRAIN) ke_planestrain(X, E, V, t, Ke);
        else ke_heat(X, E, t, Ke);
    }
}

// one thread per element of an explicit mesh: Ke_e (nk x nk) from the element's own node
// coordinates (coords: dim doubles per node), modulus E[e]
template <int KIND>
__global__ void fem_ke_kernel(long long ne, const int *__restrict__ conn, const double *__restrict__ coords,
                              const double *__restrict__ E, double V, double t, double *__restrict__ Ke) {
    constexpr int dim = KIND == PSF_H8_SOLID ? 3 : 2;
    constexpr int nd = KIND == PSF_Q4_HEAT ? 1 : dim;
    constexpr int nen = KIND == PSF_H8_SOLID ? 8 : (KIND == PSF_T3_PLANE_STRAIN ? 3 : 4);
    constexpr long long nk = (long long)nen * nd;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        double X[nen * dim];
#pragma unroll
        for (int q = 0; q < nen; q++) {
            const long long n = conn[e * nen + q];
#pragma unroll
            for (int d = 0; d < dim; d++) X[q * dim + d] = coords[n * dim + d];
        }
        double *K = Ke + e * nk * nk;
        if constexpr (KIND == PSF_H8_SOLID) {
            double wk[1008];
            ke_solid(X, E[e], V, K, wk);
        } else if constexpr (KIND == PSF_T3_PLANE_STRAIN) {
            ke_planestrain_t3(X, E[e], V, t, K);
        } else if constexpr (KIND == PSF_Q4_PLANE_STRAIN) {
            ke_planestrain(X, E[e], V, t, K);
        } else {
            ke_heat(X, E[e], t, K);
        }
    }
}

// PlaneStrainBodyForce (PlaneStrain.h:503-534) for a uniform force (fx, fy): Fe = sum_g
// B^T f J t w0 w1, B the 2 x 2nen matrix of N (T3: Gauss1Triangle, Q4: Gauss4Square)
__device__ void body_force(int kind, const double *X, double fx, double fy, double t, double *Fe) {
    const int nen = kind == PSF_T3_PLANE_STRAIN ? 3 : 4, ng = kind == PSF_T3_PLANE_STRAIN ? 1 : 4;
    for (int k = 0; k < 2 * nen; k++) Fe[k] = 0.0;
    for (int g = 0; g < ng; g++) {
        double r[2], N[4], dN[8], J2[4], w0, w1;
        if (kind == PSF_T3_PLANE_STRAIN) {
            r[0] = 1.0 / 3.0; r[1] = 1.0 / 3.0;
            N[0] = r[0]; N[1] = r[1]; N[2] = 1.0 - r[0] - r[1];
            const double d[6] = {1.0, 0.0, -1.0, 0.0, 1.0, -1.0};
            for (int k = 0; k < 6; k++) dN[k] = d[k];
            w0 = w1 = 1.0 / sqrt(2.0);
        } else {
            gauss_q4(g, r);
            N[0] = 0.25 * (1.0 - r[0]) * (1.0 - r[1]);
            N[1] = 0.25 * (1.0 + r[0]) * (1.0 - r[1]);
            N[2] = 0.25 * (1.0 + r[0]) * (1.0 + r[1]);
            N[3] = 0.25 * (1.0 - r[0]) * (1.0 + r[1]);
            dndr_q4(r, dN);
            w0 = w1 = 1.0;
        }
        mm(dN, X, J2, 2, nen, 2);
        const double J = det2(J2);
        for (int n = 0; n < nen; n++)
            for (int c = 0; c < 2; c++) {
                const double b0 = c == 0 ? N[n] : 0.0, b1 = c == 0 ? 0.0 : N[n];   // row of B^T
                double v = 0.0;
                v += b0 * fx;
                v += b1 * fy;
                Fe[2 * n + c] += v * J * t * w0 * w1;
            }
    }
}

// PlaneStrainSurfaceForce<ShapeFunction2Line, Gauss1Line> (PlaneStrain.h:421-452) for a
// uniform traction (tx, ty) on a 2-node edge: Fe = B^T f dl t w0, dl the length factor
__device__ void edge_force(const double *X, double tx, double ty, double t, double *Fe) {
    const double r = 0.0;
    const double N[2] = {0.5 * (1 - r), 0.5 * (1 + r)};
    const double dN[2] = {-0.5, 0.5};
    double d[2];
    mm(dN, X, d, 1, 2, 2);
    double q = 0.0;
    q += d[0] * d[0];
    q += d[1] * d[1];
    const double dl = sqrt(q);
    for (int k = 0; k < 4; k++) Fe[k] = 0.0;
    for (int n = 0; n < 2; n++)
        for (int c = 0; c < 2; c++) {
            const double b0 = c == 0 ? N[n] : 0.0, b1 = c == 0 ? 0.0 : N[n];
            double v = 0.0;
            v += b0 * tx;
            v += b1 * ty;
            Fe[2 * n + c] += v * dl * t * 2.0;
        }
}

__global__ void fem_body_kernel(int kind, long long ne, int nen, const int *__restrict__ conn,
                                const double *__restrict__ coords, double fx, double fy, double t,
                                double *__restrict__ Fe) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne; e += (long long)gridDim.x * blockDim.x) {
        double X[8];
        for (int q = 0; q < nen; q++)
            for (int d = 0; d < 2; d++) X[q * 2 + d] = coords[(long long)conn[e * nen + q] * 2 + d];
        body_force(kind, X, fx, fy, t, Fe + e * 2 * nen);
    }
}

__global__ void fem_edge_kernel(int nedge, const int *__restrict__ edges, const double *__restrict__ coords, double tx,
                                double ty, double t, double *__restrict__ Fe) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nedge; k += gridDim.x * blockDim.x) {
        double X[4];
        for (int q = 0; q < 2; q++)
            for (int d = 0; d < 2; d++) X[q * 2 + d] = coords[(long long)edges[2 * k + q] * 2 + d];
        edge_force(X, tx, ty, t, Fe + 4 * k);
    }
}

}  // namespace

psf_status fem_body_forces(cudaStream_t s, int kind, long long ne, int nen, const int *conn, const double *coords,
                           double fx, double fy, double t, double *Fe) {
    (fem_body_kernel<<<grid_for(ne, 128, 65536), 128, 0, s>>>(
         kind, ne, nen, conn, coords, fx, fy, t, Fe),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status fem_edge_forces(cudaStream_t s, int nedge, const int *edges, const double *coords, double tx, double ty,
                           double t, double *Fe) {
    (fem_edge_kernel<<<grid_for(nedge, 128, 65536), 128, 0, s>>>(
         nedge, edges, coords, tx, ty, t, Fe),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status fem_element_matrices(cudaStream_t s, int kind, long long ne, int nen, const int *conn, const double *coords,
                                const double *E, double V, double t, double *Ke) {
    (void)nen;
    switch (kind) {
        case PSF_Q4_PLANE_STRAIN:
            (fem_ke_kernel<PSF_Q4_PLANE_STRAIN><<<grid_for(ne, 64, 65536), 64, 0, s>>>(
                 ne, conn, coords, E, V, t, Ke),
             ::psf::note_launch());
            break;
        case PSF_Q4_HEAT:
            (fem_ke_kernel<PSF_Q4_HEAT><<<grid_for(ne, 64, 65536), 64, 0, s>>>(
                 ne, conn, coords, E, V, t, Ke),
             ::psf::note_launch());
            break;
        case PSF_H8_SOLID:
            (fem_ke_kernel<PSF_H8_SOLID><<<grid_for(ne, 64, 65536), 64, 0, s>>>(
                 ne, conn, coords, E, V, t, Ke),
             ::psf::note_launch());
            break;
        default:
            (fem_ke_kernel<PSF_T3_PLANE_STRAIN><<<grid_for(ne, 64, 65536), 64, 0, s>>>(
                 ne, conn, coords, E, V, t, Ke),
             ::psf::note_launch());
    }
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status ke_element0(Ctx *c, double E, double *Ke_dev) {
    double *wk = nullptr;
    if (c->kind == PSF_H8_SOLID) PSF_CUDA(cudaMallocAsync((void **)&wk, 576 * sizeof(double), c->stream));
    (ke_element0_kernel<<<1, 32, 0, c->stream>>>(c->kind, c->nx, c->ny, c->nz, c->lx, c->ly, c->lz, E,
                                                c->V, c->t, Ke_dev, wk), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    if (wk) PSF_CUDA(cudaFreeAsync(wk, c->stream));
    return PSF_OK;
}

}  // namespace psf
