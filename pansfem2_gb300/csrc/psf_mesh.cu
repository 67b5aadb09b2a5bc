// psf_mesh.cu -- numbering, CSR pattern, assembly, right-hand side, CSR SpMV.
//
// Everything here works on the implicit structured grid: no element list is
// stored; element e = ny*i + j (3D (ny*i + j)*nz + k) has the SquareMesh node
// order, and the element matrix is Ke0 (E = 1) scaled by E_e.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "psf_internal.cuh"

namespace psf {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
const char *last_error() { return g_last_error.c_str(); }
psf_status cuda_status(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return PSF_OK;
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return PSF_CUDA_ERROR;
}

psf_status reset_sync(Ctx *c) {
    PSF_CUDA(cudaMemsetAsync(c->gs, 0, sizeof(GridSync), c->stream));
    return PSF_OK;
}

psf_status read_sync_status(Ctx *c) {
    int st = 0;
    PSF_CUDA(cudaMemcpyAsync(&st, &c->gs->status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (st != 0) {
        set_error(st == PSF_TIMEOUT     ? "device-side grid barrier wait exceeded its limit"
                  : st == PSF_BAD_INPUT ? "zero or non-finite diagonal entry (the Jacobi scaling divides by it)"
                                        : "device-side failure in a persistent kernel");
        return (psf_status)st;
    }
    return PSF_OK;
}

psf_status launch_coop(Ctx *c, const void *fn, int blocks, int threads, void **args, size_t smem) {
    PSF_CHECK(reset_sync(c));
    PSF_CUDA(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(threads), args, smem, c->stream));
    note_launch();
    return PSF_OK;
}

// ------------------------------------------------------------------ exclusive scan (int)
namespace {
constexpr int kScanThreads = 256, kScanItems = 4, kScanTile = kScanThreads * kScanItems;

__device__ long long block_excl_scan(long long v, long long *sm, long long *total) {
    // Hillis-Steele over the block in shared memory (setup-time only)
    const int t = threadIdx.x;
    sm[t] = v;
    __syncthreads();
    for (int o = 1; o < blockDim.x; o <<= 1) {
        long long a = t >= o ? sm[t - o] : 0;
        __syncthreads();
        sm[t] += a;
        __syncthreads();
    }
    long long incl = sm[t];
    *total = sm[blockDim.x - 1];
    __syncthreads();
    return incl - v;
}

__global__ void scan_tile_sums(const int *in, long long n, long long *sums) {
    __shared__ long long sm[kScanThreads];
    long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems, v = 0;
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) v += in[base + k];
    long long tot;
    block_excl_scan(v, sm, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void scan_sums(long long *sums, int nb, long long *total) {
    // one block: sequential chunks per thread, then a block scan of the chunk totals
    __shared__ long long sm[1024];
    const int T = blockDim.x, t = threadIdx.x;
    const int chunk = (nb + T - 1) / T;
    const int b0 = t * chunk, b1 = min(nb, b0 + chunk);
    long long v = 0;
    for (int b = b0; b < b1; b++) v += sums[b];
    long long tot;
    long long off = block_excl_scan(v, sm, &tot);
    for (int b = b0; b < b1; b++) {
        long long x = sums[b];
        sums[b] = off;
        off += x;
    }
    if (t == 0) *total = tot;
}

__global__ void scan_write(const int *in, long long n, const long long *sums, int *out, int *overflow) {
    __shared__ long long sm[kScanThreads];
    long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * kScanItems, v = 0;
    int x[kScanItems];
    for (int k = 0; k < kScanItems; k++) {
        x[k] = base + k < n ? in[base + k] : 0;
        v += x[k];
    }
    long long tot;
    long long off = block_excl_scan(v, sm, &tot) + sums[blockIdx.x];
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) {
            if (off > 0x7fffffffll) *overflow = 1;
            out[base + k] = (int)off;
            off += x[k];
        }
}
}  // namespace

// out[i] = sum_{k<i} in[k] (int32 output, overflow checked); returns the total
static psf_status exclusive_scan(Ctx *c, const int *in, long long n, int *out, long long *total) {
    int nb = (int)((n + kScanTile - 1) / kScanTile);
    if (nb < 1) nb = 1;
    long long *sums = nullptr, *tot_d = nullptr;
    int *ovf = nullptr;
    PSF_CUDA(cudaMallocAsync((void **)&sums, sizeof(long long) * (nb + 1), c->stream));
    PSF_CUDA(cudaMallocAsync((void **)&ovf, sizeof(int), c->stream));
    tot_d = sums + nb;
    PSF_CUDA(cudaMemsetAsync(ovf, 0, sizeof(int), c->stream));
    (scan_tile_sums<<<nb, kScanThreads, 0, c->stream>>>(in, n, sums), ::psf::note_launch());
    (scan_sums<<<1, 1024, 0, c->stream>>>(sums, nb, tot_d), ::psf::note_launch());
    (scan_write<<<nb, kScanThreads, 0, c->stream>>>(in, n, sums, out, ovf), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    long long tot = 0;
    int o = 0;
    PSF_CUDA(cudaMemcpyAsync(&tot, tot_d, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaMemcpyAsync(&o, ovf, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaFreeAsync(sums, c->stream));
    PSF_CUDA(cudaFreeAsync(ovf, c->stream));
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    if (o || tot > 0x7fffffffll) {
        set_error("index range exceeds int32 (the reference's CSR uses int indices)");
        return PSF_BAD_INPUT;
    }
    *total = tot;
    return PSF_OK;
}

// ------------------------------------------------------------------ numbering
namespace {
__global__ void free_flags(const unsigned char *fixed, long long n, int *flag) {
    for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < n;
         a += (long long)gridDim.x * blockDim.x)
        flag[a] = fixed[a] ? 0 : 1;
}
// Renumbering (Assembling.h:175-186): running index over nodes then dofs, -1 when fixed
__global__ void write_numbering(const unsigned char *fixed, const int *prefix, long long n, int *n2g,
                                int *g2n) {
    for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < n;
         a += (long long)gridDim.x * blockDim.x) {
        if (fixed[a]) {
            n2g[a] = -1;
        } else {
            n2g[a] = prefix[a];
            g2n[prefix[a]] = (int)a;
        }
    }
}
__global__ void mark_fixed(const int *node, const int *dof, const double *val, int n, int ndof,
                           unsigned char *fixed, double *ufixed) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        long long a = (long long)node[k] * ndof + dof[k];
        fixed[a] = 1;
        ufixed[a] = val ? val[k] : 0.0;   // SetDirichlet: last writer wins, as in list order
    }
}
}  // namespace

// ------------------------------------------------------------------ grid geometry helpers
struct Grid {
    int nx, ny, nz, ndof, is3d;
    __host__ __device__ long long node_id(int i, int j, int k) const {
        return is3d ? ((long long)(ny + 1) * i + j) * (nz + 1) + k : (long long)(ny + 1) * i + j;
    }
    __host__ __device__ void node_ijk(long long n, int &i, int &j, int &k) const {
        if (is3d) {
            k = (int)(n % (nz + 1));
            long long r = n / (nz + 1);
            j = (int)(r % (ny + 1));
            i = (int)(r / (ny + 1));
        } else {
            k = 0;
            j = (int)(n % (ny + 1));
            i = (int)(n / (ny + 1));
        }
    }
    __host__ __device__ long long elem_id(int i, int j, int k) const {
        return is3d ? ((long long)ny * i + j) * nz + k : (long long)ny * i + j;
    }
    // local node index of corner offset (di, dj, dk) in {0,1}^d (SquareMesh / ShapeFunction8Cubic order)
    __host__ __device__ static int local(int di, int dj, int dk) {
        int q = di ? (dj ? 2 : 1) : (dj ? 3 : 0);
        return q + 4 * dk;
    }
};

static Grid grid_of(const Ctx *c) {
    Grid g;
    g.nx = c->nx; g.ny = c->ny; g.nz = c->nz; g.ndof = c->ndof;
    g.is3d = c->kind == PSF_H8_SOLID;
    return g;
}

struct Ke64 { double v[576]; };

namespace {
// number of free dofs in the node neighbourhood (every node sharing an element)
__global__ void pattern_count(Grid g, const int *n2g, const int *g2n, long long nfree, int *cnt) {
    for (long long I = blockIdx.x * (long long)blockDim.x + threadIdx.x; I < nfree;
         I += (long long)gridDim.x * blockDim.x) {
        long long n = g2n[I] / g.ndof;
        int i, j, k;
        g.node_ijk(n, i, j, k);
        int c = 0;
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++)
                for (int dk = g.is3d ? -1 : 0; dk <= (g.is3d ? 1 : 0); dk++) {
                    int a = i + di, b = j + dj, q = k + dk;
                    if (a < 0 || a > g.nx || b < 0 || b > g.ny || (g.is3d && (q < 0 || q > g.nz))) continue;
                    long long m = g.node_id(a, b, q);
                    for (int d = 0; d < g.ndof; d++) c += n2g[m * g.ndof + d] >= 0;
                }
        cnt[I] = c;
    }
}

// CSR(LILCSR&) (CSR.h:92-105): columns ascending.  Neighbour nodes visited in
// ascending node id and dofs ascending give ascending global numbers.
__global__ void pattern_fill(Grid g, const int *n2g, const int *g2n, long long nfree, const int *indptr,
                             int *indices, int *diag) {
    for (long long I = blockIdx.x * (long long)blockDim.x + threadIdx.x; I < nfree;
         I += (long long)gridDim.x * blockDim.x) {
        long long n = g2n[I] / g.ndof;
        int i, j, k;
        g.node_ijk(n, i, j, k);
        int o = indptr[I];
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++)
                for (int dk = g.is3d ? -1 : 0; dk <= (g.is3d ? 1 : 0); dk++) {
                    int a = i + di, b = j + dj, q = k + dk;
                    if (a < 0 || a > g.nx || b < 0 || b > g.ny || (g.is3d && (q < 0 || q > g.nz))) continue;
                    long long m = g.node_id(a, b, q);
                    for (int d = 0; d < g.ndof; d++) {
                        int J = n2g[m * g.ndof + d];
                        if (J < 0) continue;
                        if (J == (int)I) diag[I] = o;
                        indices[o++] = J;
                    }
                }
    }
}

// Assembling (Assembling.h:46-66) per row: every (I, J) entry is the sum, in
// ascending element order, of E_e * Ke0[li][lj] over the elements holding both
// nodes; the Dirichlet lift F_I -= Ke*u_fixed runs in the reference's element,
// node, dof order (skipped when every prescribed value is zero, which leaves F
// unchanged bit for bit).
template <int IS3D>
__global__ void assemble_rows(Grid g, const int *n2g, const int *g2n, long long nfree, const int *indptr,
                              const double *E, const Ke64 *Ke0, double *data, const double *ufixed,
                              int lift, double *F) {
    const int nk = (IS3D ? 8 : 4) * g.ndof;
    for (long long I = blockIdx.x * (long long)blockDim.x + threadIdx.x; I < nfree;
         I += (long long)gridDim.x * blockDim.x) {
        const long long nd = g2n[I];
        const long long n = nd / g.ndof;
        const int a = (int)(nd % g.ndof);
        int i, j, k;
        g.node_ijk(n, i, j, k);
        int o = indptr[I];
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++)
                for (int dk = IS3D ? -1 : 0; dk <= (IS3D ? 1 : 0); dk++) {
                    const int ii = i + di, jj = j + dj, kk = k + dk;
                    if (ii < 0 || ii > g.nx || jj < 0 || jj > g.ny || (IS3D && (kk < 0 || kk > g.nz))) continue;
                    const long long m = g.node_id(ii, jj, kk);
                    for (int b = 0; b < g.ndof; b++) {
                        if (n2g[m * g.ndof + b] < 0) continue;
                        double v = 0.0;
                        bool first = true;
                        // shared elements, ascending element id
                        for (int ei = max(i, ii) - 1; ei <= min(i, ii); ei++) {
                            if (ei < 0 || ei >= g.nx) continue;
                            for (int ej = max(j, jj) - 1; ej <= min(j, jj); ej++) {
                                if (ej < 0 || ej >= g.ny) continue;
                                for (int ek = IS3D ? max(k, kk) - 1 : 0; ek <= (IS3D ? min(k, kk) : 0); ek++) {
                                    if (IS3D && (ek < 0 || ek >= g.nz)) continue;
                                    const long long e = g.elem_id(ei, ej, ek);
                                    const int li = Grid::local(i - ei, j - ej, IS3D ? k - ek : 0) * g.ndof + a;
                                    const int lj = Grid::local(ii - ei, jj - ej, IS3D ? kk - ek : 0) * g.ndof + b;
                                    const double cval = E[e] * Ke0->v[li * nk + lj];
                                    v = first ? cval : v + cval;
                                    first = false;
                                }
                            }
                        }
                        data[o++] = v;
                    }
                }
        if (lift) {
            double f = F[I];
            for (int ei = i - 1; ei <= i; ei++) {
                if (ei < 0 || ei >= g.nx) continue;
                for (int ej = j - 1; ej <= j; ej++) {
                    if (ej < 0 || ej >= g.ny) continue;
                    for (int ek = IS3D ? k - 1 : 0; ek <= (IS3D ? k : 0); ek++) {
                        if (IS3D && (ek < 0 || ek >= g.nz)) continue;
                        const long long e = g.elem_id(ei, ej, ek);
                        const int li = Grid::local(i - ei, j - ej, IS3D ? k - ek : 0) * g.ndof + a;
                        for (int q = 0; q < (IS3D ? 8 : 4); q++) {
                            const int qi = (q == 1 || q == 2 || q == 5 || q == 6), qj = (q == 2 || q == 3 || q == 6 || q == 7),
                                      qk = q >= 4;
                            const long long m = g.node_id(ei + qi, ej + qj, ek + qk);
                            for (int b = 0; b < g.ndof; b++) {
                                if (n2g[m * g.ndof + b] >= 0) continue;
                                f -= E[e] * Ke0->v[li * nk + q * g.ndof + b] * ufixed[m * g.ndof + b];
                            }
                        }
                    }
                }
            }
            F[I] = f;
        }
    }
}

__global__ void loads_nodal(const int *node, const int *dof, const double *val, int n, int ndof,
                            const int *n2g, double *Fn) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) {
        long long a = (long long)node[k] * ndof + dof[k];
        if (n2g[a] >= 0) atomicAdd(&Fn[a], val[k]);
    }
}

__global__ void gather_kernel(const int *g2n, long long nfree, const double *nodal, double *red) {
    for (long long I = blockIdx.x * (long long)blockDim.x + threadIdx.x; I < nfree;
         I += (long long)gridDim.x * blockDim.x)
        red[I] = nodal[g2n[I]];
}
__global__ void scatter_kernel(const int *n2g, long long ndofs, const double *red, double *nodal) {
    for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < ndofs;
         a += (long long)gridDim.x * blockDim.x) {
        int I = n2g[a];
        nodal[a] = I >= 0 ? red[I] : 0.0;
    }
}
__global__ void add_reduced_to_nodal(const int *g2n, long long nfree, const double *red, double *nodal) {
    for (long long I = blockIdx.x * (long long)blockDim.x + threadIdx.x; I < nfree;
         I += (long long)gridDim.x * blockDim.x)
        nodal[g2n[I]] += red[I];
}

// E (ne) -> FP32 copy, zero-padded copies ((nx+2)(ny+2)[(nz+2)], element (i,j,k) at (i+1,j+1,k+1))
__global__ void moduli_pad(Grid g, long long ne, const double *E, float *Ef, double *Ep, float *Epf) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ne;
         e += (long long)gridDim.x * blockDim.x) {
        int i, j, k = 0;
        if (g.is3d) {
            k = (int)(e % g.nz);
            long long r = e / g.nz;
            j = (int)(r % g.ny);
            i = (int)(r / g.ny);
        } else {
            j = (int)(e % g.ny);
            i = (int)(e / g.ny);
        }
        long long p = g.is3d ? ((long long)(i + 1) * (g.ny + 2) + (j + 1)) * (g.nz + 2) + (k + 1)
                             : (long long)(i + 1) * (g.ny + 2) + (j + 1);
        double v = E[e];
        Ef[e] = (float)v;
        Ep[p] = v;
        Epf[p] = (float)v;
    }
}

// nodal diagonal of K: sum over the node's elements of E_e*Ke0[l,l]; 1 on fixed dofs
// nodal diagonal of K and its l1 row sums sum_j |K_ij| (the smoother's diagonal);
// 1 on fixed dofs
__global__ void nodal_diag(Grid g, long long nnodes, const double *Ep, const Ke64 *Ke0, const int *n2g,
                           double *D, float *Df, float *Dl1) {
    const int nk = (g.is3d ? 8 : 4) * g.ndof;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        g.node_ijk(n, i, j, k);
        for (int d = 0; d < g.ndof; d++) {
            double s = 0.0, s1 = 0.0;
            for (int ei = i - 1; ei <= i; ei++)
                for (int ej = j - 1; ej <= j; ej++)
                    for (int ek = g.is3d ? k - 1 : 0; ek <= (g.is3d ? k : 0); ek++) {
                        long long p = g.is3d ? ((long long)(ei + 1) * (g.ny + 2) + (ej + 1)) * (g.nz + 2) + (ek + 1)
                                             : (long long)(ei + 1) * (g.ny + 2) + (ej + 1);
                        const int l = Grid::local(i - ei, j - ej, g.is3d ? k - ek : 0) * g.ndof + d;
                        s += Ep[p] * Ke0->v[l * nk + l];
                        double rs = 0.0;
                        for (int q = 0; q < nk; q++) rs += fabs(Ke0->v[l * nk + q]);
                        s1 += Ep[p] * rs;
                    }
            long long a = n * g.ndof + d;
            if (n2g[a] < 0) { s = 1.0; s1 = 1.0; }
            D[a] = s;
            Df[a] = (float)s;
            Dl1[a] = (float)s1;
        }
    }
}

// y = A x, four threads per row (rows hold 8..81 entries), FP64
__global__ void spmv_csr64_kernel(long long rows, const int *__restrict__ indptr, const int *__restrict__ indices,
                                  const double *__restrict__ data, const double *__restrict__ x,
                                  double *__restrict__ y) {
    // the loop bound is warp-uniform (8 rows per warp) so every lane reaches the shuffles
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int sub = threadIdx.x & 3;
    const long long stride = ((long long)gridDim.x * blockDim.x) >> 2;
    for (long long base = (tid >> 5) << 3; base < rows; base += stride) {
        const long long r = base + ((threadIdx.x & 31) >> 2);
        double v = 0.0;
        if (r < rows)
            for (int q = indptr[r] + sub; q < indptr[r + 1]; q += 4) v += data[q] * x[indices[q]];
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        if (sub == 0 && r < rows) y[r] = v;
    }
}
}  // namespace

// ------------------------------------------------------------------ host entry points
psf_status set_dirichlet(Ctx *c, int n, const int *node, const int *dof, const double *value) {
    for (int k = 0; k < n; k++) {
        if (node[k] < 0 || node[k] >= c->nnodes || dof[k] < 0 || dof[k] >= c->ndof) {
            set_error("psf_set_dirichlet: (node, dof) out of range");
            return PSF_BAD_INPUT;
        }
    }
    PSF_CUDA(cudaMemsetAsync(c->fixed, 0, c->ndofs, c->stream));
    PSF_CUDA(cudaMemsetAsync(c->ufixed, 0, c->ndofs * sizeof(double), c->stream));
    c->nonzero_ufixed = false;
    if (value)
        for (int k = 0; k < n; k++)
            if (value[k] != 0.0) c->nonzero_ufixed = true;
    int *dn = nullptr, *dd = nullptr;
    double *dv = nullptr;
    if (n > 0) {
        PSF_CUDA(cudaMallocAsync((void **)&dn, sizeof(int) * n, c->stream));
        PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(int) * n, c->stream));
        PSF_CUDA(cudaMemcpyAsync(dn, node, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        PSF_CUDA(cudaMemcpyAsync(dd, dof, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        if (value) {
            PSF_CUDA(cudaMallocAsync((void **)&dv, sizeof(double) * n, c->stream));
            PSF_CUDA(cudaMemcpyAsync(dv, value, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        }
        (mark_fixed<<<grid_for(n, 256), 256, 0, c->stream>>>(
             dn, dd, dv, n, c->ndof, c->fixed, c->ufixed),
         ::psf::note_launch());
        PSF_CUDA(cudaGetLastError());
    }
    int *flag = nullptr, *prefix = nullptr;
    PSF_CUDA(cudaMallocAsync((void **)&flag, sizeof(int) * c->ndofs, c->stream));
    PSF_CUDA(cudaMallocAsync((void **)&prefix, sizeof(int) * c->ndofs, c->stream));
    (free_flags<<<grid_for(c->ndofs, 256, 65536), 256, 0, c->stream>>>(c->fixed, c->ndofs, flag), ::psf::note_launch());
    long long nfree = 0;
    PSF_CHECK(exclusive_scan(c, flag, c->ndofs, prefix, &nfree));
    c->nfree = nfree;
    if (c->g2n) { cudaFreeAsync(c->g2n, c->stream); c->g2n = nullptr; }
    PSF_CUDA(cudaMallocAsync((void **)&c->g2n, sizeof(int) * (nfree > 0 ? nfree : 1), c->stream));
    (write_numbering<<<grid_for(c->ndofs, 256, 65536), 256, 0, c->stream>>>(c->fixed, prefix, c->ndofs, c->n2g,
                                                                            c->g2n), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaFreeAsync(flag, c->stream));
    PSF_CUDA(cudaFreeAsync(prefix, c->stream));
    if (dn) PSF_CUDA(cudaFreeAsync(dn, c->stream));
    if (dd) PSF_CUDA(cudaFreeAsync(dd, c->stream));
    if (dv) PSF_CUDA(cudaFreeAsync(dv, c->stream));
    // reduced-length vectors
    for (double **p : {&c->F, &c->u}) {
        if (*p) { cudaFreeAsync(*p, c->stream); *p = nullptr; }
        PSF_CUDA(cudaMallocAsync((void **)p, sizeof(double) * (nfree > 0 ? nfree : 1), c->stream));
        PSF_CUDA(cudaMemsetAsync(*p, 0, sizeof(double) * (nfree > 0 ? nfree : 1), c->stream));
    }
    c->have_bc = true;
    c->have_csr = false;
    c->have_values = false;
    c->nnz = 0;   // the pattern depends on the fixed set: rebuilt on demand
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    return PSF_OK;
}

psf_status build_pattern(Ctx *c) {
    if (!c->have_bc) { set_error("psf_build_csr: call psf_set_dirichlet first"); return PSF_BAD_INPUT; }
    Grid g = grid_of(c);
    int *cnt = nullptr;
    if (c->indptr) { cudaFreeAsync(c->indptr, c->stream); c->indptr = nullptr; }
    if (c->diag) { cudaFreeAsync(c->diag, c->stream); c->diag = nullptr; }
    PSF_CUDA(cudaMallocAsync((void **)&cnt, sizeof(int) * (c->nfree + 1), c->stream));
    PSF_CUDA(cudaMallocAsync((void **)&c->indptr, sizeof(int) * (c->nfree + 1), c->stream));
    PSF_CUDA(cudaMallocAsync((void **)&c->diag, sizeof(int) * (c->nfree + 1), c->stream));
    PSF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (c->nfree + 1), c->stream));
    (pattern_count<<<grid_for(c->nfree, 256, 65536), 256, 0, c->stream>>>(
         g, c->n2g, c->g2n, c->nfree, cnt),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    long long nnz = 0;
    PSF_CHECK(exclusive_scan(c, cnt, c->nfree + 1, c->indptr, &nnz));
    PSF_CUDA(cudaFreeAsync(cnt, c->stream));
    c->nnz = nnz;
    if (c->indices) { cudaFreeAsync(c->indices, c->stream); c->indices = nullptr; }
    if (c->data) { cudaFreeAsync(c->data, c->stream); c->data = nullptr; }
    PSF_CUDA(cudaMallocAsync((void **)&c->indices, sizeof(int) * (nnz > 0 ? nnz : 1), c->stream));
    PSF_CUDA(cudaMallocAsync((void **)&c->data, sizeof(double) * (nnz > 0 ? nnz : 1), c->stream));
    (pattern_fill<<<grid_for(c->nfree, 256, 65536), 256, 0, c->stream>>>(g, c->n2g, c->g2n, c->nfree, c->indptr,
                                                                         c->indices, c->diag), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaStreamSynchronize(c->stream));
    c->have_csr = true;
    c->have_values = false;
    return PSF_OK;
}

psf_status build_rhs(Ctx *c) {
    // nodal point loads (Assembling.h:151-158) on free dofs
    PSF_CUDA(cudaMemsetAsync(c->Fn, 0, sizeof(double) * c->ndofs, c->stream));
    int n = (int)c->load_node.size();
    if (n > 0) {
        int *dn = nullptr, *dd = nullptr;
        double *dv = nullptr;
        PSF_CUDA(cudaMallocAsync((void **)&dn, sizeof(int) * n, c->stream));
        PSF_CUDA(cudaMallocAsync((void **)&dd, sizeof(int) * n, c->stream));
        PSF_CUDA(cudaMallocAsync((void **)&dv, sizeof(double) * n, c->stream));
        PSF_CUDA(cudaMemcpyAsync(dn, c->load_node.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        PSF_CUDA(cudaMemcpyAsync(dd, c->load_dof.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        PSF_CUDA(cudaMemcpyAsync(dv, c->load_val.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        (loads_nodal<<<grid_for(n, 256), 256, 0, c->stream>>>(
             dn, dd, dv, n, c->ndof, c->n2g, c->Fn),
         ::psf::note_launch());
        PSF_CUDA(cudaGetLastError());
        PSF_CUDA(cudaFreeAsync(dn, c->stream));
        PSF_CUDA(cudaFreeAsync(dd, c->stream));
        PSF_CUDA(cudaFreeAsync(dv, c->stream));
    }
    PSF_CHECK(gather_reduced(c, c->Fn, c->F));
    return PSF_OK;
}

psf_status set_moduli(Ctx *c, const double *E_dev) {
    if (E_dev != c->E)
        PSF_CUDA(cudaMemcpyAsync(c->E, E_dev, sizeof(double) * c->ne, cudaMemcpyDeviceToDevice, c->stream));
    Grid g = grid_of(c);
    (moduli_pad<<<grid_for(c->ne, 256, 65536), 256, 0, c->stream>>>(
         g, c->ne, c->E, c->Ef, c->Epad, c->Epadf),
     ::psf::note_launch());
    (nodal_diag<<<grid_for(c->nnodes, 256, 65536), 256, 0, c->stream>>>(g, c->nnodes, c->Epad, (const Ke64 *)c->Ke0,
                                                                         c->n2g, c->Dn, c->Dnf, c->Dl1f),
                                                                         ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status assemble_values(Ctx *c, const double *E_dev) {
    if (!c->have_csr) PSF_CHECK(build_pattern(c));
    PSF_CHECK(set_moduli(c, E_dev));
    PSF_CHECK(build_rhs(c));
    Grid g = grid_of(c);
    const int lift = c->nonzero_ufixed ? 1 : 0;
    if (g.is3d)
        (assemble_rows<1><<<grid_for(c->nfree, 128, 65536), 128, 0, c->stream>>>(
            g, c->n2g, c->g2n, c->nfree, c->indptr, c->E, (const Ke64 *)c->Ke0, c->data, c->ufixed, lift, c->F),
            ::psf::note_launch());
    else
        (assemble_rows<0><<<grid_for(c->nfree, 128, 65536), 128, 0, c->stream>>>(
            g, c->n2g, c->g2n, c->nfree, c->indptr, c->E, (const Ke64 *)c->Ke0, c->data, c->ufixed, lift, c->F),
            ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    c->have_values = true;
    return PSF_OK;
}

psf_status spmv_csr64(Ctx *c, const double *x, double *y) {
    (spmv_csr64_kernel<<<grid_for(c->nfree * 4, 256, c->num_sms * 16), 256, 0, c->stream>>>(
        c->nfree, c->indptr, c->indices, c->data, x, y), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status gather_reduced(Ctx *c, const double *nodal, double *red) {
    (gather_kernel<<<grid_for(c->nfree, 256, 65536), 256, 0, c->stream>>>(
         c->g2n, c->nfree, nodal, red),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status scatter_reduced(Ctx *c, const double *red, double *nodal) {
    (scatter_kernel<<<grid_for(c->ndofs, 256, 65536), 256, 0, c->stream>>>(
         c->n2g, c->ndofs, red, nodal),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

}  // namespace psf
