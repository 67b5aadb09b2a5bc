// psf_fem.cu -- explicit (unstructured) meshes: the reference's general assembly path.
//
// A mesh is node coordinates plus element connectivity, as ImportFromCSV.h:22-98 reads
// them or a sample writes them out (sample/planestrain/sample_planestrain.cpp:20-23).  On
// the device, per call:
//   * element matrices from each element's own coordinates (psf_element.cu: T3 / Q4 plane
//     strain, Q4 heat, H8 solid, bit for bit the reference's routines);
//   * SetDirichlet + Renumbering (BoundaryCondition.h:19-25, Assembling.h:175-186): free dofs
//     numbered node-major, dof-minor;
//   * Assembling into LILCSR, then CSR(LILCSR&) (Assembling.h:46-66, CSR.h:92-105): the pattern
//     is every free-free pair sharing an element (exact zeros included), columns ascending;
//     each entry sums its element contributions from 0.0 in ascending element order (one
//     thread per node builds the node's sorted neighbour list once, then walks the node's
//     elements in that order for each of its rows), so the values equal the reference's bit
//     for bit; F[I] -= Ke u_fixed and the uniform body force
//     (PlaneStrainBodyForce) in the same order, then the point loads in list order
//     (Assembling.h:151-158), then uniform edge tractions (PlaneStrainSurfaceForce);
//   * the solve on the CSR (CG.h solvers of psf_solve.cu) and the reaction
//     r = sum_e Ke_e u_e over all dofs (the samples' RemoveBoundaryConditions + Renumbering +
//     Assembling of Ke*ElementVector, sample_planestrain.cpp:66-77).
// Node-to-element lists are built with atomics and then sorted, so every order is fixed.
#include <algorithm>
#include <vector>

#include "psf_internal.cuh"

namespace psf {
psf_status pcg_csr_any(Ctx *c, long long rows, const int *indptr, const int *indices, const int *diag,
                       const double *data, const double *b, double *x, double *w, int jacobi, int itmax, double eps,
                       int *iters, double *rr, double *bb, int *conv);  // psf_solve.cu
psf_status generic_context(Ctx **out);                                   // psf_generic.cu

namespace {

constexpr int kMaxNb = 96;   // distinct nodes sharing an element with one node (Q4 9, H8 27)

__global__ void adj_count(long long ne, int nen, const int *__restrict__ conn, int *__restrict__ cnt) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ne * nen; t += (long long)gridDim.x * blockDim.x)
        atomicAdd(&cnt[conn[t]], 1);
}
__global__ void adj_fill(long long ne, int nen, const int *__restrict__ conn, const int *__restrict__ ptr,
                         int *__restrict__ pos, int *__restrict__ adj) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ne * nen; t += (long long)gridDim.x * blockDim.x) {
        const int n = conn[t];
        adj[ptr[n] + atomicAdd(&pos[n], 1)] = (int)(t / nen);
    }
}
// each node's element list in ascending element id (insertion sort; lists are short)
__global__ void adj_sort(long long nn, const int *__restrict__ ptr, int *__restrict__ adj) {
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < nn; n += (long long)gridDim.x * blockDim.x) {
        for (int a = ptr[n] + 1; a < ptr[n + 1]; a++) {
            const int v = adj[a];
            int b = a - 1;
            while (b >= ptr[n] && adj[b] > v) {
                adj[b + 1] = adj[b];
                b--;
            }
            adj[b + 1] = v;
        }
    }
}

// exclusive scan of n ints (one block per 1024 entries, then the block sums, then the offsets)
__global__ void scan_blocks(long long n, const int *__restrict__ in, int *__restrict__ out, int *__restrict__ bsum) {
    __shared__ int s[1024];
    const long long i = blockIdx.x * 1024LL + threadIdx.x;
    s[threadIdx.x] = i < n ? in[i] : 0;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = threadIdx.x >= o ? s[threadIdx.x - o] : 0;
        __syncthreads();
        s[threadIdx.x] += v;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - (i < n ? in[i] : 0);
    if (threadIdx.x == 1023) bsum[blockIdx.x] = s[1023];
}
__global__ void scan_sums(int nb, int *__restrict__ bsum, int *__restrict__ total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int b = 0; b < nb; b++) {
        const int v = bsum[b];
        bsum[b] = acc;
        acc += v;
    }
    *total = acc;
}
__global__ void scan_add(long long n, int *__restrict__ out, const int *__restrict__ bsum) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] += bsum[i / 1024];
}

__global__ void mark_fixed_kernel(int n, const int *__restrict__ node, const int *__restrict__ dof,
                                  const double *__restrict__ val, int nd, unsigned char *__restrict__ fixed,
                                  double *__restrict__ ufix) {
    // list order: a later entry for the same dof wins, as SetDirichlet's loop does
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int k = 0; k < n; k++) {
        const long long t = (long long)node[k] * nd + dof[k];
        fixed[t] = 1;
        ufix[t] = val ? val[k] : 0.0;
    }
}
__global__ void free_flags_kernel(long long nt, const unsigned char *__restrict__ fixed, int *__restrict__ f) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += (long long)gridDim.x * blockDim.x)
        f[t] = fixed[t] ? 0 : 1;
}
__global__ void numbering_kernel(long long nt, const unsigned char *__restrict__ fixed, int *__restrict__ n2g) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += (long long)gridDim.x * blockDim.x)
        if (fixed[t]) n2g[t] = -1;
}

struct MeshArgs {
    int nen, nd, nk;
    long long nn;
    const int *conn, *adj_ptr, *adj, *n2g;
    const unsigned char *fixed;
};

// The nodes that share an element with node n, ascending, without repeats; false when there
// are more than kMaxNb.  Renumbering (Assembling.h:175-186) numbers the free dofs node-major
// and dof-minor, so the free dofs of these nodes, taken in this order, are the sorted distinct
// columns of every row of node n: the rows of one node share one column list.
template <int MAXNB>
__device__ bool node_neighbours(const MeshArgs &M, long long n, int *nb, int &cnt) {
    cnt = 0;
    for (int p = M.adj_ptr[n]; p < M.adj_ptr[n + 1]; p++) {
        const long long e = M.adj[p];
        for (int j = 0; j < M.nen; j++) {
            const int m = M.conn[e * M.nen + j];
            int k = cnt;   // insertion into the sorted list, skipping repeats
            while (k > 0 && nb[k - 1] > m) k--;
            if (k > 0 && nb[k - 1] == m) continue;
            if (cnt >= MAXNB) return false;
            for (int q = cnt; q > k; q--) nb[q] = nb[q - 1];
            nb[k] = m;
            cnt++;
        }
    }
    return true;
}

// one thread per node: the number of columns of each of its free rows
__global__ void pattern_count_kernel(MeshArgs M, int *__restrict__ cnt, int *__restrict__ err) {
    int nb[kMaxNb];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < M.nn; n += (long long)gridDim.x * blockDim.x) {
        bool any = false;
        for (int a = 0; a < M.nd; a++) any = any || M.n2g[n * M.nd + a] >= 0;
        if (!any) continue;
        int k = 0;
        if (!node_neighbours<kMaxNb>(M, n, nb, k)) { atomicExch(err, 1); continue; }
        int nc = 0;
        for (int q = 0; q < k; q++)
            for (int b = 0; b < M.nd; b++) nc += M.n2g[(long long)nb[q] * M.nd + b] >= 0;
        for (int a = 0; a < M.nd; a++) {
            const int I = M.n2g[n * M.nd + a];
            if (I >= 0) cnt[I] = nc;
        }
    }
}

// first position of key in the ascending list a[0..n), n when absent
__device__ __forceinline__ int first_of(const int *__restrict__ a, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// indices, values (element contributions from 0.0 in ascending element order), F (per
// element in that order its fixed-dof terms and its body force, then the point loads in list
// order, then the edge tractions in edge order: the sample's sequence), diagonal position
// The per-node lists are per-thread arrays (local memory, L1-cached).  Keeping one row's values
// in shared memory instead, interleaved across the block's threads, was slower: 1.2-1.5 ms
// against 1.0 ms at 1M dofs, with fewer resident warps for this latency-bound walk.
__global__ void assemble_rows_kernel(MeshArgs M, const double *__restrict__ Ke, const double *__restrict__ ufix,
                                     int nload, const int *__restrict__ lnode, const int *__restrict__ ldof,
                                     const double *__restrict__ lval, const double *__restrict__ Fbody, int nedge,
                                     const int *__restrict__ enode, const int *__restrict__ eslot,
                                     const double *__restrict__ Fedge, const int *__restrict__ indptr,
                                     int *__restrict__ indices, double *__restrict__ data, double *__restrict__ F,
                                     int *__restrict__ diag, int *__restrict__ err) {
    int nb[kMaxNb], off[kMaxNb + 1];
    double vals[kMaxNb * 3];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < M.nn; n += (long long)gridDim.x * blockDim.x) {
        bool any = false;
        for (int a = 0; a < M.nd; a++) any = any || M.n2g[n * M.nd + a] >= 0;
        if (!any) continue;
        int k = 0;
        if (!node_neighbours<kMaxNb>(M, n, nb, k)) { atomicExch(err, 1); continue; }
        off[0] = 0;   // first column of each neighbour's free dofs
        for (int q = 0; q < k; q++) {
            int c = 0;
            for (int b = 0; b < M.nd; b++) c += M.n2g[(long long)nb[q] * M.nd + b] >= 0;
            off[q + 1] = off[q] + c;
        }
        const int nc = off[k];
        for (int a = 0; a < M.nd; a++) {   // the rows of node n, one after the other
            const int I = M.n2g[n * M.nd + a];
            if (I < 0) continue;
            for (int c = 0; c < nc; c++) vals[c] = 0.0;
            double f = 0.0;
            for (int p = M.adj_ptr[n]; p < M.adj_ptr[n + 1]; p++) {   // ascending element order
                const long long e = M.adj[p];
                int i = 0;
                while (i < M.nen && M.conn[e * M.nen + i] != n) i++;
                const double *K = Ke + e * (long long)M.nk * M.nk + (long long)(i * M.nd + a) * M.nk;
                for (int j = 0; j < M.nen; j++) {
                    const int m = M.conn[e * M.nen + j];
                    int lo = 0, hi = k;   // m's place among the neighbours
                    while (lo < hi) {
                        const int mid = (lo + hi) >> 1;
                        if (nb[mid] < m) lo = mid + 1;
                        else hi = mid;
                    }
                    int c = off[lo];
                    for (int b = 0; b < M.nd; b++) {
                        const long long u = (long long)m * M.nd + b;
                        const double kv = K[j * M.nd + b];
                        if (M.n2g[u] >= 0) {
                            vals[c] = __dadd_rn(vals[c], kv);
                            c++;
                        } else {
                            f = __dsub_rn(f, __dmul_rn(kv, ufix[u]));
                        }
                    }
                }
                if (Fbody) f = __dadd_rn(f, Fbody[e * M.nk + i * M.nd + a]);   // the element's body force
            }
            // point loads, then edge tractions: both lists are sorted by node, stably, so a
            // node's entries keep their list (edge) order
            for (int l = first_of(lnode, nload, (int)n); l < nload && lnode[l] == n; l++)
                if (ldof[l] == a) f = __dadd_rn(f, lval[l]);
            for (int l = first_of(enode, 2 * nedge, (int)n); l < 2 * nedge && enode[l] == n; l++)
                f = __dadd_rn(f, Fedge[eslot[l] + a]);
            const int base = indptr[I];
            int dg = -1, c = 0;
            for (int q = 0; q < k; q++)
                for (int b = 0; b < M.nd; b++) {
                    const int J = M.n2g[(long long)nb[q] * M.nd + b];
                    if (J < 0) continue;
                    indices[base + c] = J;
                    data[base + c] = vals[c];
                    if (J == I) dg = base + c;
                    c++;
                }
            diag[I] = dg;
            F[I] = f;
        }
    }
}

// nodal u from the reduced solution (free dofs) and the prescribed values (fixed dofs)
__global__ void scatter_u_kernel(long long nt, const int *__restrict__ n2g, const double *__restrict__ x,
                                 const double *__restrict__ ufix, double *__restrict__ u) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nt; t += (long long)gridDim.x * blockDim.x)
        u[t] = n2g[t] >= 0 ? x[n2g[t]] : ufix[t];
}

// r(dof) = sum over the node's elements (ascending) of (Ke_e u_e)(local row), each row a dot
// product from 0.0 in column order (Matrix * Vector), every dof numbered
__global__ void reaction_kernel(MeshArgs M, const double *__restrict__ Ke, const double *__restrict__ u,
                                double *__restrict__ r) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M.nn * M.nd;
         t += (long long)gridDim.x * blockDim.x) {
        const long long n = t / M.nd;
        const int a = (int)(t % M.nd);
        double acc = 0.0;
        for (int p = M.adj_ptr[n]; p < M.adj_ptr[n + 1]; p++) {
            const long long e = M.adj[p];
            int i = 0;
            while (i < M.nen && M.conn[e * M.nen + i] != n) i++;
            const double *K = Ke + e * (long long)M.nk * M.nk + (long long)(i * M.nd + a) * M.nk;
            double row = 0.0;
            for (int j = 0; j < M.nen; j++) {
                const long long m = M.conn[e * M.nen + j];
                for (int b = 0; b < M.nd; b++) row = __dadd_rn(row, __dmul_rn(K[j * M.nd + b], u[m * M.nd + b]));
            }
            acc = __dadd_rn(acc, row);
        }
        r[t] = acc;
    }
}

}  // namespace

struct FemMesh {
    int kind = 0, nen = 0, nd = 0, dim = 0, nk = 0;
    long long nn = 0, ne = 0;
    int *conn = nullptr, *adj_ptr = nullptr, *adj = nullptr;
    double *coords = nullptr, *E = nullptr, *Ke = nullptr;
    unsigned char *fixed = nullptr;
    double *ufix = nullptr;
    int *n2g = nullptr, nfree = 0;
    bool have_bc = false, have_sys = false;
    int *indptr = nullptr, *indices = nullptr, *diag = nullptr;
    double *data = nullptr, *F = nullptr;
    long long nnz = 0;
    int nload = 0;
    int *lnode = nullptr, *ldof = nullptr;
    double *lval = nullptr;
    bool body = false;
    double bfx = 0.0, bfy = 0.0;
    double *Fbody = nullptr;       // ne x nk
    int nedge = 0;
    int *edges = nullptr;
    int *enode = nullptr, *eslot = nullptr;   // edge ends sorted by node: node, 4 k + 2 q
    double etx = 0.0, ety = 0.0;
    double *Fedge = nullptr;       // nedge x 4
    size_t cap_indptr = 0, cap_indices = 0, cap_data = 0, cap_diag = 0, cap_F = 0;   // bytes held
    // scratch kept between calls (a cudaFree waits for the whole device)
    enum { kScrCnt, kScrBs, kScrTot, kScrErr, kScrDn, kScrDd, kScrDv, kScrFlags, kScrN };
    void *scr[kScrN] = {};
    size_t scr_cap[kScrN] = {};
    std::vector<void *> allocs;
    Ctx *c = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};   // phases of the last assembly
    double ms[3] = {0.0, 0.0, 0.0};                             // element matrices, pattern, values
};

static psf_status fem_alloc(FemMesh *f, void **p, size_t bytes) {
    PSF_CUDA(cudaMalloc(p, bytes ? bytes : 1));
    f->allocs.push_back(*p);
    return PSF_OK;
}
static void fem_release(FemMesh *f, void *p) {
    if (!p) return;
    cudaFree(p);
    f->allocs.erase(std::remove(f->allocs.begin(), f->allocs.end(), p), f->allocs.end());
}

// *p holds at least `bytes` (its contents are not kept when it grows)
template <class T>
static psf_status fem_reserve(FemMesh *f, T **p, size_t *cap, size_t bytes) {
    if (*p && *cap >= bytes) return PSF_OK;
    fem_release(f, *p);
    *p = nullptr;
    *cap = 0;
    PSF_CHECK(fem_alloc(f, (void **)p, bytes));
    *cap = bytes;
    return PSF_OK;
}
template <class T>
static psf_status fem_scratch(FemMesh *f, int slot, size_t bytes, T **out) {
    PSF_CHECK(fem_reserve(f, &f->scr[slot], &f->scr_cap[slot], bytes));
    *out = (T *)f->scr[slot];
    return PSF_OK;
}

// exclusive scan of n device ints into out; the total into *total (host)
static psf_status scan_ints(FemMesh *f, long long n, const int *in, int *out, int *total) {
    const long long nb = (n + 1023) / 1024;
    int *bs = nullptr, *tot = nullptr;
    PSF_CHECK(fem_scratch(f, FemMesh::kScrBs, sizeof(int) * (nb + 1), &bs));
    PSF_CHECK(fem_scratch(f, FemMesh::kScrTot, sizeof(int), &tot));
    cudaStream_t s = f->c->stream;
    if (nb > 0) (scan_blocks<<<(unsigned)nb, 1024, 0, s>>>(n, in, out, bs), ::psf::note_launch());
    (scan_sums<<<1, 32, 0, s>>>((int)nb, bs, tot), ::psf::note_launch());
    if (nb > 0) (scan_add<<<grid_for(n, 256, 65536), 256, 0, s>>>(n, out, bs), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(total, tot, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    return PSF_OK;
}

static MeshArgs mesh_args(const FemMesh *f) {
    MeshArgs M;
    M.nen = f->nen; M.nd = f->nd; M.nk = f->nk; M.nn = f->nn;
    M.conn = f->conn; M.adj_ptr = f->adj_ptr; M.adj = f->adj; M.n2g = f->n2g; M.fixed = f->fixed;
    return M;
}

}  // namespace psf

using psf::FemMesh;

struct psf_fem {
    FemMesh m;
};

#define FEM_CHECK(h)                                                         \
    do {                                                                     \
        if (!(h)) { psf::set_error("psf_fem: null mesh"); return PSF_BAD_INPUT; } \
    } while (0)

extern "C" {

psf_status psf_fem_create(int kind, long long nnodes, const double *coords, long long nelem, int nen,
                          const int32_t *conn, psf_fem **out) {
    using namespace psf;
    if (!out || !coords || !conn || nnodes <= 0 || nelem <= 0) { set_error("psf_fem_create: invalid arguments"); return PSF_BAD_INPUT; }
    const int want = kind == PSF_T3_PLANE_STRAIN ? 3 : (kind == PSF_H8_SOLID ? 8 : 4);
    if (kind < 0 || kind > 3 || nen != want) { set_error("psf_fem_create: kind / nodes per element mismatch"); return PSF_BAD_INPUT; }
    for (long long t = 0; t < nelem * nen; t++)
        if (conn[t] < 0 || conn[t] >= nnodes) { set_error("psf_fem_create: connectivity out of range"); return PSF_BAD_INPUT; }
    if (nnodes * 3 > 0x7fffffffLL) { set_error("psf_fem_create: mesh too large"); return PSF_BAD_INPUT; }
    psf_fem *h = new psf_fem;
    FemMesh *f = &h->m;
    f->kind = kind; f->nen = nen; f->nn = nnodes; f->ne = nelem;
    f->dim = kind == PSF_H8_SOLID ? 3 : 2;
    f->nd = kind == PSF_Q4_HEAT ? 1 : f->dim;
    f->nk = nen * f->nd;
    psf_status st = generic_context(&f->c);
    auto A = [&](psf_status s) { if (st == PSF_OK) st = s; };
    A(fem_alloc(f, (void **)&f->conn, sizeof(int) * nelem * nen));
    A(fem_alloc(f, (void **)&f->coords, sizeof(double) * nnodes * f->dim));
    A(fem_alloc(f, (void **)&f->E, sizeof(double) * nelem));
    A(fem_alloc(f, (void **)&f->Ke, sizeof(double) * nelem * f->nk * f->nk));
    A(fem_alloc(f, (void **)&f->adj_ptr, sizeof(int) * (nnodes + 1)));
    A(fem_alloc(f, (void **)&f->adj, sizeof(int) * nelem * nen));
    A(fem_alloc(f, (void **)&f->fixed, nnodes * f->nd));
    A(fem_alloc(f, (void **)&f->ufix, sizeof(double) * nnodes * f->nd));
    A(fem_alloc(f, (void **)&f->n2g, sizeof(int) * nnodes * f->nd));
    for (auto &e : f->ev) A(cuda_status(cudaEventCreate(&e), "event"));
    int *cnt = nullptr, *pos = nullptr;
    A(fem_alloc(f, (void **)&cnt, sizeof(int) * (nnodes + 1)));
    A(fem_alloc(f, (void **)&pos, sizeof(int) * (nnodes + 1)));
    if (st == PSF_OK) {
        cudaStream_t s = f->c->stream;
        A(cuda_status(cudaMemcpyAsync(f->conn, conn, sizeof(int) * nelem * nen, cudaMemcpyHostToDevice, s), "copy"));
        A(cuda_status(cudaMemcpyAsync(f->coords, coords, sizeof(double) * nnodes * f->dim, cudaMemcpyHostToDevice, s),
                      "copy"));
        A(cuda_status(cudaMemsetAsync(cnt, 0, sizeof(int) * (nnodes + 1), s), "memset"));
        A(cuda_status(cudaMemsetAsync(pos, 0, sizeof(int) * (nnodes + 1), s), "memset"));
        A(cuda_status(cudaMemsetAsync(f->fixed, 0, nnodes * f->nd, s), "memset"));
        A(cuda_status(cudaMemsetAsync(f->ufix, 0, sizeof(double) * nnodes * f->nd, s), "memset"));
        if (st == PSF_OK) {
            (adj_count<<<grid_for(nelem * nen, 256, 65536), 256, 0, s>>>(
                 nelem, nen, f->conn, cnt),
             ::psf::note_launch());
            int total = 0;
            A(scan_ints(f, nnodes + 1, cnt, f->adj_ptr, &total));
            (adj_fill<<<grid_for(nelem * nen, 256, 65536), 256, 0, s>>>(
                 nelem, nen, f->conn, f->adj_ptr, pos, f->adj),
             ::psf::note_launch());
            (adj_sort<<<grid_for(nnodes, 256, 65536), 256, 0, s>>>(nnodes, f->adj_ptr, f->adj), ::psf::note_launch());
            A(cuda_status(cudaGetLastError(), "adjacency"));
        }
    }
    fem_release(f, cnt);
    fem_release(f, pos);
    if (st != PSF_OK) {
        for (void *p : f->allocs) cudaFree(p);
        for (auto e : f->ev)
            if (e) cudaEventDestroy(e);
        delete h;
        return st;
    }
    *out = h;
    return PSF_OK;
}

psf_status psf_fem_destroy(psf_fem *h) {
    if (!h) return PSF_OK;
    cudaStreamSynchronize(h->m.c->stream);
    for (void *p : h->m.allocs) cudaFree(p);
    for (auto e : h->m.ev)
        if (e) cudaEventDestroy(e);
    delete h;
    return PSF_OK;
}

psf_status psf_fem_set_dirichlet(psf_fem *h, int n, const int32_t *node, const int32_t *dof, const double *value,
                                 int *nfree) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    for (int k = 0; k < n; k++)
        if (node[k] < 0 || node[k] >= f->nn || dof[k] < 0 || dof[k] >= f->nd) {
            set_error("psf_fem_set_dirichlet: node or dof out of range");
            return PSF_BAD_INPUT;
        }
    cudaStream_t s = f->c->stream;
    const long long nt = f->nn * f->nd;
    int *dn = nullptr, *dd = nullptr, *flags = nullptr;
    double *dv = nullptr;
    PSF_CHECK(fem_scratch(f, FemMesh::kScrDn, sizeof(int) * (n + 1), &dn));
    PSF_CHECK(fem_scratch(f, FemMesh::kScrDd, sizeof(int) * (n + 1), &dd));
    PSF_CHECK(fem_scratch(f, FemMesh::kScrDv, sizeof(double) * (n + 1), &dv));
    PSF_CHECK(fem_scratch(f, FemMesh::kScrFlags, sizeof(int) * nt, &flags));
    PSF_CUDA(cudaMemsetAsync(f->fixed, 0, nt, s));
    PSF_CUDA(cudaMemsetAsync(f->ufix, 0, sizeof(double) * nt, s));
    if (n > 0) {
        PSF_CUDA(cudaMemcpyAsync(dn, node, sizeof(int) * n, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaMemcpyAsync(dd, dof, sizeof(int) * n, cudaMemcpyHostToDevice, s));
        if (value) PSF_CUDA(cudaMemcpyAsync(dv, value, sizeof(double) * n, cudaMemcpyHostToDevice, s));
        (mark_fixed_kernel<<<1, 32, 0, s>>>(
             n, dn, dd, value ? dv : nullptr, f->nd, f->fixed, f->ufix),
         ::psf::note_launch());
    }
    (free_flags_kernel<<<grid_for(nt, 256, 65536), 256, 0, s>>>(nt, f->fixed, flags), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    int total = 0;
    PSF_CHECK(scan_ints(f, nt, flags, f->n2g, &total));
    (numbering_kernel<<<grid_for(nt, 256, 65536), 256, 0, s>>>(nt, f->fixed, f->n2g), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaStreamSynchronize(s));
    f->nfree = total;
    f->have_bc = true;
    f->have_sys = false;
    if (nfree) *nfree = total;
    return PSF_OK;
}

psf_status psf_fem_set_loads(psf_fem *h, int n, const int32_t *node, const int32_t *dof, const double *value) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (n < 0 || (n > 0 && (!node || !dof || !value))) { set_error("psf_fem_set_loads: invalid arrays"); return PSF_BAD_INPUT; }
    for (int k = 0; k < n; k++)
        if (node[k] < 0 || node[k] >= f->nn || dof[k] < 0 || dof[k] >= f->nd) {
            set_error("psf_fem_set_loads: (node, dof) out of range");
            return PSF_BAD_INPUT;
        }
    // sorted by node, stably: the assembly walks a node's loads in list order
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return node[x] < node[y]; });
    std::vector<int> sn(n), sd(n);
    std::vector<double> sv(n);
    for (int k = 0; k < n; k++) { sn[k] = node[order[k]]; sd[k] = dof[order[k]]; sv[k] = value[order[k]]; }
    for (void *p : {(void *)f->lnode, (void *)f->ldof, (void *)f->lval}) fem_release(f, p);
    f->lnode = nullptr; f->ldof = nullptr; f->lval = nullptr;
    PSF_CHECK(fem_alloc(f, (void **)&f->lnode, sizeof(int) * (n + 1)));
    PSF_CHECK(fem_alloc(f, (void **)&f->ldof, sizeof(int) * (n + 1)));
    PSF_CHECK(fem_alloc(f, (void **)&f->lval, sizeof(double) * (n + 1)));
    cudaStream_t s = f->c->stream;
    if (n > 0) {
        PSF_CUDA(cudaMemcpyAsync(f->lnode, sn.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaMemcpyAsync(f->ldof, sd.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaMemcpyAsync(f->lval, sv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    }
    PSF_CUDA(cudaStreamSynchronize(s));
    f->nload = n;
    return PSF_OK;
}

psf_status psf_fem_set_body_force(psf_fem *h, double fx, double fy) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (f->kind != PSF_Q4_PLANE_STRAIN && f->kind != PSF_T3_PLANE_STRAIN) {
        set_error("psf_fem_set_body_force: plane-strain meshes only");
        return PSF_BAD_INPUT;
    }
    f->body = true;
    f->bfx = fx;
    f->bfy = fy;
    return PSF_OK;
}

psf_status psf_fem_set_edge_loads(psf_fem *h, int nedge, const int32_t *edges, double tx, double ty) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (f->kind != PSF_Q4_PLANE_STRAIN && f->kind != PSF_T3_PLANE_STRAIN) {
        set_error("psf_fem_set_edge_loads: plane-strain meshes only");
        return PSF_BAD_INPUT;
    }
    if (nedge < 0 || (nedge > 0 && !edges)) { set_error("psf_fem_set_edge_loads: invalid edges"); return PSF_BAD_INPUT; }
    for (int k = 0; k < 2 * nedge; k++)
        if (edges[k] < 0 || edges[k] >= f->nn) { set_error("psf_fem_set_edge_loads: node out of range"); return PSF_BAD_INPUT; }
    for (void *p : {(void *)f->edges, (void *)f->Fedge, (void *)f->enode, (void *)f->eslot}) fem_release(f, p);
    f->edges = nullptr;
    f->Fedge = nullptr;
    f->enode = nullptr;
    f->eslot = nullptr;
    f->nedge = nedge;
    f->etx = tx;
    f->ety = ty;
    if (nedge > 0) {
        // the edge ends sorted by node, stably, so a node's tractions keep the edge order
        std::vector<int> order(2 * (size_t)nedge), en(2 * (size_t)nedge), es(2 * (size_t)nedge);
        for (int k = 0; k < 2 * nedge; k++) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return edges[x] < edges[y]; });
        for (int k = 0; k < 2 * nedge; k++) { en[k] = edges[order[k]]; es[k] = 2 * order[k]; }   // 4 e + 2 q
        PSF_CHECK(fem_alloc(f, (void **)&f->edges, sizeof(int) * 2 * nedge));
        PSF_CHECK(fem_alloc(f, (void **)&f->enode, sizeof(int) * 2 * nedge));
        PSF_CHECK(fem_alloc(f, (void **)&f->eslot, sizeof(int) * 2 * nedge));
        cudaStream_t s = f->c->stream;
        PSF_CUDA(cudaMemcpyAsync(f->edges, edges, sizeof(int) * 2 * nedge, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaMemcpyAsync(f->enode, en.data(), sizeof(int) * 2 * nedge, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaMemcpyAsync(f->eslot, es.data(), sizeof(int) * 2 * nedge, cudaMemcpyHostToDevice, s));
        PSF_CUDA(cudaStreamSynchronize(s));
    }
    return PSF_OK;
}

psf_status psf_fem_assemble(psf_fem *h, const double *E, double V, double t, long long *nnz) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (!E) { set_error("psf_fem_assemble: null moduli"); return PSF_BAD_INPUT; }
    if (!f->have_bc) { set_error("psf_fem_assemble: call psf_fem_set_dirichlet first"); return PSF_BAD_INPUT; }
    cudaStream_t s = f->c->stream;
    PSF_CUDA(cudaMemcpyAsync(f->E, E, sizeof(double) * f->ne, cudaMemcpyHostToDevice, s));
    PSF_CUDA(cudaEventRecord(f->ev[0], s));
    PSF_CHECK(fem_element_matrices(s, f->kind, f->ne, f->nen, f->conn, f->coords, f->E, V, t, f->Ke));
    PSF_CUDA(cudaEventRecord(f->ev[1], s));
    const MeshArgs M = mesh_args(f);
    int *err = nullptr;
    PSF_CHECK(fem_scratch(f, FemMesh::kScrErr, sizeof(int), &err));
    PSF_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    if (!f->have_sys) {   // pattern: counts per free row, then the row pointers
        int *cnt = nullptr;
        PSF_CHECK(fem_scratch(f, FemMesh::kScrCnt, sizeof(int) * (f->nfree + 1), &cnt));
        PSF_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (f->nfree + 1), s));
        (pattern_count_kernel<<<grid_for(f->nn, 128, 65536), 128, 0, s>>>(M, cnt, err), ::psf::note_launch());
        PSF_CUDA(cudaGetLastError());
        PSF_CHECK(fem_reserve(f, &f->indptr, &f->cap_indptr, sizeof(int) * (f->nfree + 1)));
        int total = 0;
        PSF_CHECK(scan_ints(f, f->nfree + 1, cnt, f->indptr, &total));
        f->nnz = total;
        PSF_CHECK(fem_reserve(f, &f->indices, &f->cap_indices, sizeof(int) * (f->nnz + 1)));
        PSF_CHECK(fem_reserve(f, &f->data, &f->cap_data, sizeof(double) * (f->nnz + 1)));
        PSF_CHECK(fem_reserve(f, &f->diag, &f->cap_diag, sizeof(int) * (f->nfree + 1)));
        PSF_CHECK(fem_reserve(f, &f->F, &f->cap_F, sizeof(double) * (f->nfree + 1)));
    }
    PSF_CUDA(cudaEventRecord(f->ev[2], s));
    if (f->body) {
        if (!f->Fbody) PSF_CHECK(fem_alloc(f, (void **)&f->Fbody, sizeof(double) * f->ne * f->nk));
        PSF_CHECK(fem_body_forces(s, f->kind, f->ne, f->nen, f->conn, f->coords, f->bfx, f->bfy, t, f->Fbody));
    }
    if (f->nedge > 0) {
        if (!f->Fedge) PSF_CHECK(fem_alloc(f, (void **)&f->Fedge, sizeof(double) * 4 * f->nedge));
        PSF_CHECK(fem_edge_forces(s, f->nedge, f->edges, f->coords, f->etx, f->ety, t, f->Fedge));
    }
    (assemble_rows_kernel<<<grid_for(f->nn, 128, 65536), 128, 0, s>>>(
         M, f->Ke, f->ufix, f->nload, f->lnode, f->ldof, f->lval, f->body ? f->Fbody : nullptr, f->nedge, f->enode,
         f->eslot, f->Fedge, f->indptr, f->indices, f->data, f->F, f->diag, err),
     ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaEventRecord(f->ev[3], s));
    int herr = 0;
    PSF_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < 3; k++) {
        float ms = 0.0f;
        PSF_CUDA(cudaEventElapsedTime(&ms, f->ev[k], f->ev[k + 1]));
        f->ms[k] = ms;
    }
    if (herr) {
        set_error("psf_fem_assemble: a node shares elements with more than 96 other nodes");
        return PSF_BAD_INPUT;
    }
    f->have_sys = true;
    if (nnz) *nnz = f->nnz;
    return PSF_OK;
}

psf_status psf_fem_timings(psf_fem *h, double *element_ms, double *pattern_ms, double *values_ms) {
    using namespace psf;
    FEM_CHECK(h);
    if (!h->m.have_sys) { set_error("psf_fem_timings: assemble first"); return PSF_BAD_INPUT; }
    if (element_ms) *element_ms = h->m.ms[0];
    if (pattern_ms) *pattern_ms = h->m.ms[1];
    if (values_ms) *values_ms = h->m.ms[2];
    return PSF_OK;
}

psf_status psf_fem_get_system(psf_fem *h, int32_t *n2g, int32_t *indptr, int32_t *indices, double *data,
                              double *F) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (!f->have_sys) { set_error("psf_fem_get_system: assemble first"); return PSF_BAD_INPUT; }
    cudaStream_t s = f->c->stream;
    if (n2g) PSF_CUDA(cudaMemcpyAsync(n2g, f->n2g, sizeof(int) * f->nn * f->nd, cudaMemcpyDeviceToHost, s));
    if (indptr) PSF_CUDA(cudaMemcpyAsync(indptr, f->indptr, sizeof(int) * (f->nfree + 1), cudaMemcpyDeviceToHost, s));
    if (indices) PSF_CUDA(cudaMemcpyAsync(indices, f->indices, sizeof(int) * f->nnz, cudaMemcpyDeviceToHost, s));
    if (data) PSF_CUDA(cudaMemcpyAsync(data, f->data, sizeof(double) * f->nnz, cudaMemcpyDeviceToHost, s));
    if (F) PSF_CUDA(cudaMemcpyAsync(F, f->F, sizeof(double) * f->nfree, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    return PSF_OK;
}

psf_status psf_fem_solve(psf_fem *h, int solver, int itmax, double eps, double *u_nodal, psf_solve_info *info) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (!f->have_sys || !u_nodal) { set_error("psf_fem_solve: assemble first / null output"); return PSF_BAD_INPUT; }
    if (solver != PSF_SOLVE_CSR_JACOBI_F64 && solver != PSF_SOLVE_CSR_CG_F64) {
        set_error("psf_fem_solve: solver must be CSR_JACOBI_F64 (ScalingCG) or CSR_CG_F64 (CG)");
        return PSF_BAD_INPUT;
    }
    Ctx *c = f->c;
    cudaStream_t s = c->stream;
    const long long n = f->nfree, nt = f->nn * f->nd;
    double *x = nullptr, *w = nullptr, *u = nullptr;
    PSF_CHECK(fem_alloc(f, (void **)&x, sizeof(double) * (n + 1)));
    PSF_CHECK(fem_alloc(f, (void **)&w, sizeof(double) * 7 * (n + 1)));   // the CSR PCG's workspace
    PSF_CHECK(fem_alloc(f, (void **)&u, sizeof(double) * nt));
    c->ksec = 0.0;
    c->klaunch = 0;
    int it = 0, conv = 0;
    double rr = 0.0, bb = 0.0;
    psf_status st = pcg_csr_any(c, n, f->indptr, f->indices, f->diag, f->data, f->F, x, w,
                                solver == PSF_SOLVE_CSR_JACOBI_F64 ? 1 : 0, itmax, eps, &it, &rr, &bb, &conv);
    if (st == PSF_OK) {
        (scatter_u_kernel<<<grid_for(nt, 256, 65536), 256, 0, s>>>(nt, f->n2g, x, f->ufix, u), ::psf::note_launch());
        st = cuda_status(cudaGetLastError(), "scatter");
    }
    if (st == PSF_OK) st = cuda_status(cudaMemcpyAsync(u_nodal, u, sizeof(double) * nt, cudaMemcpyDeviceToHost, s), "copy");
    cudaStreamSynchronize(s);
    for (void *p : {(void *)x, (void *)w, (void *)u}) fem_release(f, p);
    if (st != PSF_OK) return st;
    if (info) {
        psf_solve_info inf{};
        inf.iterations = it;
        inf.outer_iterations = 1;
        inf.rel_residual_recurrence = bb > 0 ? sqrt(rr / bb) : 0.0;
        inf.rel_residual = -1.0;
        inf.kernel_seconds = c->ksec;
        inf.kernel_launches = c->klaunch;
        *info = inf;
    }
    return conv ? PSF_OK : PSF_NOT_CONVERGED;
}

psf_status psf_fem_reaction(psf_fem *h, const double *u_nodal, double *r_nodal) {
    using namespace psf;
    FEM_CHECK(h);
    FemMesh *f = &h->m;
    if (!u_nodal || !r_nodal) { set_error("psf_fem_reaction: null array"); return PSF_BAD_INPUT; }
    if (!f->have_sys) { set_error("psf_fem_reaction: assemble first"); return PSF_BAD_INPUT; }
    cudaStream_t s = f->c->stream;
    const long long nt = f->nn * f->nd;
    double *u = nullptr, *r = nullptr;
    PSF_CHECK(fem_alloc(f, (void **)&u, sizeof(double) * nt));
    PSF_CHECK(fem_alloc(f, (void **)&r, sizeof(double) * nt));
    PSF_CUDA(cudaMemcpyAsync(u, u_nodal, sizeof(double) * nt, cudaMemcpyHostToDevice, s));
    (reaction_kernel<<<grid_for(nt, 128, 65536), 128, 0, s>>>(mesh_args(f), f->Ke, u, r), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(r_nodal, r, sizeof(double) * nt, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    fem_release(f, u);
    fem_release(f, r);
    return PSF_OK;
}

}  // extern "C"
