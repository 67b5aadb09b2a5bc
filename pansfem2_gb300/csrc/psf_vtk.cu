// psf_vtk.cu -- legacy VTK output of one design iteration, the per-iteration
// dump of the reference samples (sample_optimize_density_oc.cpp:173-181 with
// ExportToVTK.h:19-141): points, cells, cell types, point vectors "u" and "r"
// (the reaction K u over all dofs), cell scalars "s" (the filtered density).
//
// The reaction is one matrix-free pass on the device; the three fields are
// copied to pinned host buffers in stream order, and the file is written by a
// host thread that waits for that copy, so the next SIMP iteration can start
// at once.  The text is produced with the same iostream formatting as the
// reference writer (default precision, tab separators).
#include <fstream>
#include <string>
#include <thread>

#include "psf_ebe.cuh"
#include "psf_internal.cuh"

namespace psf {

struct VtkState {
    double *d_r = nullptr;                      // device reaction (nodal)
    double *h_rho = nullptr, *h_u = nullptr, *h_r = nullptr;   // pinned
    cudaEvent_t copied = nullptr;
    std::thread writer;
    psf_status last = PSF_OK;
    std::string last_msg;
};

// r = K u over every dof (fixed rows included): the support reactions and, on the free dofs, K u
template <int KIND>
__global__ void reaction_kernel(Geo g, KeT<double> Ke, const double *__restrict__ Ep, const double *__restrict__ u,
                                double *__restrict__ r) {
    constexpr int nd = ndof_of<KIND>();
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < g.nnodes;
         n += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        node_ijk<KIND>(g, n, i, j, k);
        double y[nd];
        ebe_node<double, KIND>(g, Ke, Ep, i, j, k, [&](long long a) { return u[a]; }, y);
#pragma unroll
        for (int a = 0; a < nd; a++) r[n * nd + a] = y[a];
    }
}

static void write_vtk_file(const Ctx *c, const std::string &path, const double *rho, const double *u,
                           const double *r, VtkState *V) {
    std::ofstream f(path);
    if (!f) {
        V->last = PSF_BAD_INPUT;
        V->last_msg = "psf_export_vtk: cannot open " + path;
        return;
    }
    const bool is3d = c->kind == PSF_H8_SOLID;
    const int nd = c->ndof;
    f << "# vtk DataFile Version 4.1\n";
    f << "vtk output\n";
    f << "ASCII\n";
    f << "DATASET UNSTRUCTURED_GRID\n";
    // points: x = lx * (i / nx) (SquareMesh.h / CubeMesh.h), padded to 3 components
    f << "\nPOINTS\t" << c->nnodes << "\tfloat\n";
    for (int i = 0; i <= c->nx; i++)
        for (int j = 0; j <= c->ny; j++)
            for (int k = 0; k <= (is3d ? c->nz : 0); k++) {
                f << c->lx * (i / (double)c->nx) << "\t" << c->ly * (j / (double)c->ny) << "\t";
                if (is3d)
                    f << c->lz * (k / (double)c->nz) << "\t";
                else
                    f << 0.0 << "\t";
                f << std::endl;
            }
    const int nen = is3d ? 8 : 4;
    f << "\nCELLS " << c->ne << "\t" << c->ne * (nen + 1) << "\n";
    auto nid = [c, is3d](int i, int j, int k) -> long long {
        return is3d ? ((long long)(c->ny + 1) * i + j) * (c->nz + 1) + k : (long long)(c->ny + 1) * i + j;
    };
    for (int i = 0; i < c->nx; i++)
        for (int j = 0; j < c->ny; j++)
            for (int k = 0; k < (is3d ? c->nz : 1); k++) {
                f << nen << "\t";
                const int nk = is3d ? 2 : 1;
                for (int q = 0; q < nk; q++)
                    f << nid(i, j, k + q) << "\t" << nid(i + 1, j, k + q) << "\t" << nid(i + 1, j + 1, k + q) << "\t"
                      << nid(i, j + 1, k + q) << "\t";
                f << std::endl;
            }
    f << "\nCELL_TYPES\t" << c->ne << "\n";
    for (long long e = 0; e < c->ne; e++) f << (is3d ? 12 : 9) << "\n";
    auto vectors = [&](const double *v, const char *name, bool header) {
        if (header) f << "\nPOINT_DATA\t" << c->nnodes << "\n";
        f << "VECTORS " << name << " float\n";
        for (long long n = 0; n < c->nnodes; n++) {
            int a = 0;
            for (; a < nd; a++) f << v[n * nd + a] << "\t";
            for (; a < 3; a++) f << 0.0 << "\t";
            f << std::endl;
        }
    };
    vectors(u, "u", true);
    vectors(r, "r", false);
    f << "\nCELL_DATA\t" << c->ne << "\n";
    f << "SCALARS s float\n";
    f << "LOOKUP_TABLE default\n";
    for (long long e = 0; e < c->ne; e++) f << rho[e] << std::endl;
    if (!f) {
        V->last = PSF_BAD_INPUT;
        V->last_msg = "psf_export_vtk: write failed for " + path;
    }
}

static psf_status vtk_wait(Ctx *c) {
    VtkState *V = (VtkState *)c->vtk;
    if (!V) return PSF_OK;
    if (V->writer.joinable()) V->writer.join();
    if (V->last != PSF_OK) {
        set_error(V->last_msg);
        psf_status s = V->last;
        V->last = PSF_OK;
        return s;
    }
    return PSF_OK;
}

void vtk_free(Ctx *c) {
    VtkState *V = (VtkState *)c->vtk;
    if (!V) return;
    if (V->writer.joinable()) V->writer.join();
    if (V->d_r) cudaFree(V->d_r);
    if (V->h_rho) cudaFreeHost(V->h_rho);
    if (V->h_u) cudaFreeHost(V->h_u);
    if (V->h_r) cudaFreeHost(V->h_r);
    if (V->copied) cudaEventDestroy(V->copied);
    delete V;
    c->vtk = nullptr;
}

psf_status export_vtk(Ctx *c, const char *path, int async) {
    if (!path || !*path) {
        set_error("psf_export_vtk: empty path");
        return PSF_BAD_INPUT;
    }
    if (!c->simp_ready) {
        set_error("psf_export_vtk: no design (psf_simp_begin)");
        return PSF_BAD_INPUT;
    }
    PSF_CHECK(vtk_wait(c));
    if (!c->vtk) {
        VtkState *V = new VtkState();
        c->vtk = V;
        PSF_CUDA(cudaMalloc(&V->d_r, sizeof(double) * c->ndofs));
        PSF_CUDA(cudaMallocHost(&V->h_rho, sizeof(double) * c->ne));
        PSF_CUDA(cudaMallocHost(&V->h_u, sizeof(double) * c->ndofs));
        PSF_CUDA(cudaMallocHost(&V->h_r, sizeof(double) * c->ndofs));
        PSF_CUDA(cudaEventCreateWithFlags(&V->copied, cudaEventDisableTiming));
    }
    VtkState *V = (VtkState *)c->vtk;
    Geo g;
    g.nx = c->nx;
    g.ny = c->ny;
    g.nz = c->nz;
    g.nnodes = c->nnodes;
    KeT<double> Ke{};
    const int nk = c->nen * c->ndof;
    for (int q = 0; q < nk * nk; q++) Ke.v[q] = c->Ke0_host[q];
    const int grid = grid_for(c->nnodes, 256, 4 * std::max(c->num_sms, 1));
    switch (c->kind) {
        case PSF_Q4_PLANE_STRAIN:
            (reaction_kernel<PSF_Q4_PLANE_STRAIN><<<grid, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->un, V->d_r),
             ::psf::note_launch());
            break;
        case PSF_Q4_HEAT:
            (reaction_kernel<PSF_Q4_HEAT><<<grid, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->un, V->d_r),
             ::psf::note_launch());
            break;
        default:
            (reaction_kernel<PSF_H8_SOLID><<<grid, 256, 0, c->stream>>>(
                 g, Ke, c->Epad, c->un, V->d_r),
             ::psf::note_launch());
            break;
    }
    PSF_CUDA(cudaGetLastError());
    PSF_CUDA(cudaMemcpyAsync(V->h_rho, c->rho, sizeof(double) * c->ne, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaMemcpyAsync(V->h_u, c->un, sizeof(double) * c->ndofs, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaMemcpyAsync(V->h_r, V->d_r, sizeof(double) * c->ndofs, cudaMemcpyDeviceToHost, c->stream));
    PSF_CUDA(cudaEventRecord(V->copied, c->stream));
    const std::string p(path);
    auto job = [c, p, V]() {
        if (cudaEventSynchronize(V->copied) != cudaSuccess) {
            V->last = PSF_CUDA_ERROR;
            V->last_msg = "psf_export_vtk: device copy failed";
            return;
        }
        write_vtk_file(c, p, V->h_rho, V->h_u, V->h_r, V);
    };
    if (async) {
        V->writer = std::thread(job);
        return PSF_OK;
    }
    job();
    return vtk_wait(c);
}

}  // namespace psf

extern "C" {

psf_status psf_export_vtk(psf_ctx *h, const char *path, int async) {
    if (!h) return PSF_BAD_INPUT;
    return psf::export_vtk(&h->c, path, async);
}

psf_status psf_export_wait(psf_ctx *h) {
    if (!h) return PSF_BAD_INPUT;
    return psf::vtk_wait(&h->c);
}

}  // extern "C"
