// psf_unet.cu -- the network of the learned preconditioner: a 4-level U-Net on
// the vertex-centred node grid of a structured mesh, bf16 weights and
// activations with fp32 accumulation, trained on the GPU by these kernels.
//
// Convolutions (3x3, stride 1 or 2, and the transposed forms the backward pass
// needs) are implicit GEMMs on the 5th-generation tensor cores: one CTA of 128
// threads computes an 8 x 16-pixel x N-channel tile whose fp32 accumulator lives in
// tensor memory.  Each thread stages its pixel's im2col row (64 K values per
// chunk) into shared memory in the no-swizzle K-major core-matrix layout, the
// weights arrive pre-packed in the same layout, one thread issues four
// tcgen05.mma (K = 16 each) per chunk and commits them to the chunk's mbarrier
// (two stages; the loads of chunk s+1 go out into registers while chunk s is
// stored and its MMAs issued), and the
// epilogue reads the accumulator with tcgen05.ld, adds the bias, applies ReLU
// and stores bf16 (or fp32, optionally accumulating, for gradients).  Every
// mbarrier wait is bounded (about one second), after which the kernel records
// an error and returns.
//
// Weight gradients are fp32 reductions over pixels on the CUDA cores (bf16
// inputs, fp32 accumulation, fixed-order partial sums: deterministic).
//
// Network layout (the CPU oracle oracle/unet_oracle.c restates it):
//   tensors  0 input(8: density, residual x/y, 4 element moduli, 1 zero)  1 e0a  2 cat0 = [e0 | up(d1)]
//            3 e1a  4 cat1 = [e1 | up(d2)]  5 e2a  6 cat2 = [e2 | up(e3)]  7 e3a  8 e3
//            9 d2a 10 d2 11 d1a 12 d1 13 d0a 14 d0 15 output (2, fp32)
//   channels c0, 2c0, 4c0, 8c0 on levels 0..3; level sizes H_l = (H_{l-1} + 1) / 2
//   parameters per layer: W[co][tap][ci] then b[co], tap = 3*dy + dx for offset (dy-1, dx-1)
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "psf_common.cuh"
#include "psf_unet.cuh"

namespace psf {
namespace unet {

// ------------------------------------------------------------------ layer table
int layer_table(int c0, LayerDesc *L) {
    const int c1 = 2 * c0, c2 = 4 * c0, c3 = 8 * c0;
    const LayerDesc t[kLayers] = {
        // cin, cout, stride, relu, level, in, in_cs, in_c0, out, out_cs, out_c0
        {8, c0, 1, 1, 0, 0, 8, 0, 1, c0, 0, 0, 0},
        {c0, c0, 1, 1, 0, 1, c0, 0, 2, c0 + c1, 0, 0, 0},
        {c0, c1, 2, 1, 1, 2, c0 + c1, 0, 3, c1, 0, 0, 0},
        {c1, c1, 1, 1, 1, 3, c1, 0, 4, c1 + c2, 0, 0, 0},
        {c1, c2, 2, 1, 2, 4, c1 + c2, 0, 5, c2, 0, 0, 0},
        {c2, c2, 1, 1, 2, 5, c2, 0, 6, c2 + c3, 0, 0, 0},
        {c2, c3, 2, 1, 3, 6, c2 + c3, 0, 7, c3, 0, 0, 0},
        {c3, c3, 1, 1, 3, 7, c3, 0, 8, c3, 0, 0, 0},
        {c2 + c3, c2, 1, 1, 2, 6, c2 + c3, 0, 9, c2, 0, 0, 0},
        {c2, c2, 1, 1, 2, 9, c2, 0, 10, c2, 0, 0, 0},
        {c1 + c2, c1, 1, 1, 1, 4, c1 + c2, 0, 11, c1, 0, 0, 0},
        {c1, c1, 1, 1, 1, 11, c1, 0, 12, c1, 0, 0, 0},
        {c0 + c1, c0, 1, 1, 0, 2, c0 + c1, 0, 13, c0, 0, 0, 0},
        {c0, c0, 1, 1, 0, 13, c0, 0, 14, c0, 0, 0, 0},
        {c0, 2, 1, 0, 0, 14, c0, 0, 15, 2, 0, 0, 0},
    };
    int off = 0;
    for (int l = 0; l < kLayers; l++) {
        L[l] = t[l];
        L[l].woff = off;
        off += L[l].cout * 9 * L[l].cin;
        L[l].boff = off;
        off += L[l].cout;
    }
    return off;
}

void tensor_shape(int c0, int *C, int *lev) {
    const int c1 = 2 * c0, c2 = 4 * c0, c3 = 8 * c0;
    const int Ct[kTensors] = {8, c0, c0 + c1, c1, c1 + c2, c2, c2 + c3, c3, c3, c2, c2, c1, c1, c0, c0, 2};
    const int lt[kTensors] = {0, 0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0};
    for (int i = 0; i < kTensors; i++) {
        C[i] = Ct[i];
        lev[i] = lt[i];
    }
}

static inline int pad16(int c) { return (c + 15) / 16 * 16; }

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t s_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t cnt) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(cnt) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase of the given parity: false after ~2^31 cycles (~1 s)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try(bar, parity)) {
        if (clock64() - t0 > (1ll << 31)) return false;
    }
    return true;
}
__device__ __forceinline__ void tc_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 TMEM lanes (this warp's quarter) x 16 consecutive 32-bit columns
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// shared-memory matrix descriptor, no swizzle: start, leading (K-direction)
// and stride (M/N-direction) byte offsets between 8x16-byte core matrices
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor: fp32 accumulator, bf16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ------------------------------------------------------------------ convolution (implicit GEMM)
template <int N>
struct ConvSmem {
    static constexpr int A = 128 * 64 * 2;  // 128 rows x 64 K values, bf16
    static constexpr int B = N * 64 * 2;
    static constexpr int STAGE = A + B;
    static constexpr int BYTES = 2 * STAGE + 64;
    static constexpr uint32_t COLS = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
};

// input pixel of output (oy, ox) for tap offset (dy, dx) in {-1,0,1}^2
__device__ __forceinline__ bool tap_src(int mode, int oy, int ox, int dy, int dx, int hin, int win, int &yi, int &xi) {
    switch (mode) {
        case kFwdS1: yi = oy + dy; xi = ox + dx; break;
        case kFwdS2: yi = 2 * oy + dy; xi = 2 * ox + dx; break;
        case kBwdS1: yi = oy - dy; xi = ox - dx; break;
        default: {
            const int ty = oy - dy, tx = ox - dx;
            if ((ty | tx) & 1) return false;
            yi = ty >> 1;
            xi = tx >> 1;
        }
    }
    return yi >= 0 && yi < hin && xi >= 0 && xi < win;
}

constexpr int kTileH = 8, kTileW = 16;   // output pixels of a CTA's tile (128 = the MMA's M)
constexpr int kTapGroups = 512;          // 8-wide K groups in the per-CTA (tap, channel) table
constexpr int kConvCarveout = 75;

template <int N>
__global__ void __launch_bounds__(128) conv_mma_kernel(const __grid_constant__ ConvArgs a) {
    using S = ConvSmem<N>;
    extern __shared__ __align__(128) uint8_t smem[];
    if (a.skip && *a.skip) return;
    const int tid = threadIdx.x, warp = tid >> 5;
    uint8_t *meta = smem + 2 * S::STAGE;
    const uint32_t sbase = s_addr(smem);
    const uint32_t bar0 = s_addr(meta), bar1 = bar0 + 8, slot = bar0 + 16;
    if (warp == 0) tc_alloc(slot, S::COLS);
    if (tid == 0) {
        mbar_init(bar0, 1);
        mbar_init(bar1, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(meta + 16);

    // the CTA's tile: kTileH x kTileW output pixels of one image (2D, so that the 3x3 taps of
    // the tile's pixels share a small halo in L1); thread tid takes pixel (tid / kTileW,
    // tid % kTileW) of it, rows past the image edge are zero and not stored
    const int tiles_x = (a.wout + kTileW - 1) / kTileW, tiles_y = (a.hout + kTileH - 1) / kTileH;
    long long tq = blockIdx.x;
    const int tx = (int)(tq % tiles_x);
    tq /= tiles_x;
    const int ty = (int)(tq % tiles_y);
    const int b = (int)(tq / tiles_y);
    const int oy = ty * kTileH + tid / kTileW, ox = tx * kTileW + tid % kTileW;
    const bool pv = oy < a.hout && ox < a.wout;
    const long long p = ((long long)b * a.hout + oy) * a.wout + ox;
    const bf16 *xb = a.x + (size_t)b * a.hin * a.win * a.x_cs + a.x_c0;
    const int K = 9 * a.cin;
    constexpr uint32_t IDESC = idesc_bf16(128, N);
    // (tap, channel) of each 8-wide K group, computed once per CTA: the gathers then need no
    // integer division (layers of up to kTapGroups / 8 chunks; wider ones divide inline)
    __shared__ uint32_t s_tap[kTapGroups];
    const bool tab = a.nchunks * 8 <= kTapGroups;
    if (tab) {
        for (int gi = tid; gi < a.nchunks * 8; gi += 128) {
            const int k = gi * 8, tap = k / a.cin;
            s_tap[gi] = (uint32_t)tap | ((uint32_t)(k - tap * a.cin) << 4);
        }
        __syncthreads();
    }
    // The next chunks are loaded into registers while chunk s is stored and its MMAs issued, so
    // the L2 round trips of the gathers (A and B together) overlap the rest of the steps.
    // A: this thread's row, 8 core-matrix columns of 8 K values (one tap, 8 channels each);
    // B: the packed chunk, already in core-matrix order, N / 16 uint4 per thread.
    constexpr int kBPer = N / 16;
    // register sets in flight: two for the narrow layers (chunk s + 2 loads while chunk s is
    // stored), one where two sets of B would cost too many registers
    constexpr int kAhead = N <= 64 ? 2 : 1;
    uint4 ra[kAhead][8], rb[kAhead][kBPer];
    auto load_chunk = [&](int s, uint4(&va)[8], uint4(&vb)[kBPer]) {
#pragma unroll
        for (int kc = 0; kc < 8; kc++) {
            const int k = s * 64 + kc * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (pv && k < K) {
                int tap, ci;
                if (tab) {
                    const uint32_t e = s_tap[s * 8 + kc];
                    tap = (int)(e & 15u);
                    ci = (int)(e >> 4);
                } else {
                    tap = k / a.cin;
                    ci = k - tap * a.cin;
                }
                int yi, xi;
                if (tap_src(a.mode, oy, ox, tap / 3 - 1, tap % 3 - 1, a.hin, a.win, yi, xi))
                    v = __ldg(reinterpret_cast<const uint4 *>(xb + ((size_t)yi * a.win + xi) * a.x_cs + ci));
            }
            va[kc] = v;
        }
        const uint4 *wsrc = reinterpret_cast<const uint4 *>(a.w + (size_t)s * N * 64);
#pragma unroll
        for (int j = 0; j < kBPer; j++) vb[j] = __ldg(wsrc + tid + 128 * j);
    };
    bool ok = true;
    int issued = 0;   // chunks whose MMAs were issued (the same in every thread)
    // chunk s: wait for the MMAs of chunk s - 2 (its stage), store its registers, send out the
    // loads of chunk s + kAhead into the same registers, then one thread issues the MMAs
    auto step = [&](int s, uint4(&va)[8], uint4(&vb)[kBPer]) {
        const int st = s & 1;
        uint8_t *As = smem + st * S::STAGE;
        uint8_t *Bs = As + S::A;
        if (s >= 2) ok = mbar_wait(st ? bar1 : bar0, ((s >> 1) - 1) & 1) && ok;
#pragma unroll
        for (int kc = 0; kc < 8; kc++) *reinterpret_cast<uint4 *>(As + (kc * 128 + tid) * 16) = va[kc];
#pragma unroll
        for (int j = 0; j < kBPer; j++) reinterpret_cast<uint4 *>(Bs)[tid + 128 * j] = vb[j];
        if (s + kAhead < a.nchunks) load_chunk(s + kAhead, va, vb);
        fence_async_smem();
        ok = __syncthreads_and(ok) != 0;
        if (!ok) return;
        issued = s + 1;
        if (tid == 0) {
            tc_fence_after();
            const uint32_t a0 = sbase + st * S::STAGE, b0 = a0 + S::A;
#pragma unroll
            for (int kk = 0; kk < 4; kk++) {
                const uint64_t ad = sdesc(a0 + kk * 2 * 128 * 16, 128 * 16, 128);
                const uint64_t bd = sdesc(b0 + kk * 2 * N * 16, N * 16, 128);
                tc_mma(tmem, ad, bd, IDESC, (s > 0 || kk > 0) ? 1u : 0u);
            }
            tc_commit(st ? bar1 : bar0);
        }
    };
#pragma unroll
    for (int h = 0; h < kAhead; h++)
        if (h < a.nchunks) load_chunk(h, ra[h], rb[h]);
    for (int s = 0; s < a.nchunks && ok; s += kAhead) {
#pragma unroll
        for (int h = 0; h < kAhead; h++) {
            if (s + h >= a.nchunks || !ok) break;
            step(s + h, ra[h], rb[h]);
        }
    }
    if (ok) {
        const int s = a.nchunks - 1;
        ok = mbar_wait((s & 1) ? bar1 : bar0, (s >> 1) & 1);
    }
    ok = __syncthreads_and(ok) != 0;
    tc_fence_after();
    if (ok) {
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int c = 0; c < N; c += 16) {
            float v[16];
            tc_ld16(trow + c, v);
            if (!pv || c >= a.cstore) continue;
            if (a.bias) {
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] += __ldg(a.bias + c + j);
            }
            if (a.relu) {
#pragma unroll
                for (int j = 0; j < 16; j++) v[j] = fmaxf(v[j], 0.0f);
            }
            if (a.y) {
                uint4 o[2];
                uint32_t *ow = reinterpret_cast<uint32_t *>(o);
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
                    ow[j] = *reinterpret_cast<uint32_t *>(&h);
                }
                uint4 *dst = reinterpret_cast<uint4 *>(a.y + (size_t)p * a.y_cs + a.y_c0 + c);
                dst[0] = o[0];
                dst[1] = o[1];
            } else {
                float *dst = a.y32 + (size_t)p * a.y_cs + a.y_c0 + c;
                const int n = min(16, a.cstore - c);
#pragma unroll
                for (int j = 0; j < 16; j++)
                    if (j < n) dst[j] = (a.accumulate ? dst[j] : 0.0f) + v[j];
            }
        }
    } else {
        if (tid == 0) atomicExch(a.err, 1);
        // a wait gave up: wait (bounded again) for the MMAs already issued before TMEM is freed
        if (issued > 0) mbar_wait(((issued - 1) & 1) ? bar1 : bar0, ((issued - 1) >> 1) & 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, S::COLS);
}

template <int N>
static cudaError_t launch_conv_n(const ConvArgs &a, cudaStream_t st) {
    using S = ConvSmem<N>;
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(conv_mma_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, S::BYTES);
        if (e != cudaSuccess) return e;
        // shared-memory share of the unified L1 (percent; PSF_CONV_CARVEOUT overrides): fewer
        // resident CTAs but more L1 for the tap gathers.  A learned FCG solve at 1025 x 513
        // nodes took 22.3 ms with 75, 25.1 with the CUDA driver's default and with 100, 30.2 with 50.
        const char *cv = getenv("PSF_CONV_CARVEOUT");
        e = cudaFuncSetAttribute(conv_mma_kernel<N>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cv && *cv ? atoi(cv) : kConvCarveout);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const long long tiles = (long long)a.batch * ((a.hout + kTileH - 1) / kTileH) * ((a.wout + kTileW - 1) / kTileW);
    const unsigned grid = (unsigned)tiles;
    if (grid == 0) return cudaSuccess;
    (conv_mma_kernel<N><<<grid, 128, S::BYTES, st>>>(a), ::psf::note_launch());
    return cudaGetLastError();
}

// the dynamic shared-memory opt-in of every instantiation (called before any stream capture)
cudaError_t conv_init_attrs() {
    const int Ns[7] = {16, 32, 48, 64, 96, 128, 192};
    for (int N : Ns) {
        ConvArgs a{};
        a.batch = 0;   // empty launch: only sets the attribute
        cudaError_t e = cudaSuccess;
        switch (N) {
            case 16: e = launch_conv_n<16>(a, 0); break;
            case 32: e = launch_conv_n<32>(a, 0); break;
            case 48: e = launch_conv_n<48>(a, 0); break;
            case 64: e = launch_conv_n<64>(a, 0); break;
            case 96: e = launch_conv_n<96>(a, 0); break;
            case 128: e = launch_conv_n<128>(a, 0); break;
            default: e = launch_conv_n<192>(a, 0); break;
        }
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_conv(int N, const ConvArgs &a, cudaStream_t st) {
    switch (N) {
        case 16: return launch_conv_n<16>(a, st);
        case 32: return launch_conv_n<32>(a, st);
        case 48: return launch_conv_n<48>(a, st);
        case 64: return launch_conv_n<64>(a, st);
        case 96: return launch_conv_n<96>(a, st);
        case 128: return launch_conv_n<128>(a, st);
        case 192: return launch_conv_n<192>(a, st);
        default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------------------ weight packing
// forward: B[n = co][k = tap*cin + ci]; backward (data gradient): B[n = ci][k = tap*coutp + co].
// Output order per 64-wide K chunk s: [kc 0..7][n 0..N-1][e 0..7], k = 64 s + 8 kc + e.
__global__ void pack_kernel(const float *__restrict__ W, int cout, int cin, int N, int kin, int nchunks, int bwd,
                            bf16 *__restrict__ out) {
    const long long total = (long long)nchunks * 64 * N;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx & 7);
        const int n = (int)((idx >> 3) % N);
        const long long r = idx / (8ll * N);
        const int kc = (int)(r & 7);
        const int s = (int)(r >> 3);
        const int k = s * 64 + kc * 8 + e;
        float v = 0.0f;
        if (k < 9 * kin) {
            const int tap = k / kin, j = k - tap * kin;
            if (!bwd) {
                if (n < cout) v = W[((size_t)n * 9 + tap) * cin + j];  // co = n, ci = j
            } else {
                if (j < cout && n < cin) v = W[((size_t)j * 9 + tap) * cin + n];  // co = j, ci = n
            }
        }
        out[idx] = __float2bfloat16_rn(v);
    }
}

// ------------------------------------------------------------------ elementwise pieces
// bilinear vertex prolongation: fine channels [dc0, dc0 + C) of dst from the coarse tensor src (C channels)
__global__ void upsample_kernel(const bf16 *__restrict__ src, int C, int hc, int wc, bf16 *__restrict__ dst, int dcs,
                                int dc0, int hf, int wf, int batch, const int *skip) {
    if (skip && *skip) return;
    const int groups = C / 8;
    const long long total = (long long)batch * hf * wf * groups;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int g = (int)(idx % groups);
        long long q = idx / groups;
        const int x = (int)(q % wf);
        q /= wf;
        const int y = (int)(q % hf);
        const int b = (int)(q / hf);
        const int y0 = y >> 1, y1 = (y + 1) >> 1, x0 = x >> 1, x1 = (x + 1) >> 1;
        const bf16 *sb = src + (size_t)b * hc * wc * C + g * 8;
        const uint4 u00 = *reinterpret_cast<const uint4 *>(sb + ((size_t)y0 * wc + x0) * C);
        const uint4 u01 = *reinterpret_cast<const uint4 *>(sb + ((size_t)y0 * wc + x1) * C);
        const uint4 u10 = *reinterpret_cast<const uint4 *>(sb + ((size_t)y1 * wc + x0) * C);
        const uint4 u11 = *reinterpret_cast<const uint4 *>(sb + ((size_t)y1 * wc + x1) * C);
        const bf16 *h00 = reinterpret_cast<const bf16 *>(&u00), *h01 = reinterpret_cast<const bf16 *>(&u01);
        const bf16 *h10 = reinterpret_cast<const bf16 *>(&u10), *h11 = reinterpret_cast<const bf16 *>(&u11);
        uint4 o;
        bf16 *ho = reinterpret_cast<bf16 *>(&o);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float s = (__bfloat162float(h00[j]) + __bfloat162float(h01[j])) +
                            (__bfloat162float(h10[j]) + __bfloat162float(h11[j]));
            ho[j] = __float2bfloat16_rn(0.25f * s);
        }
        *reinterpret_cast<uint4 *>(dst + (((size_t)b * hf + y) * wf + x) * dcs + dc0 + g * 8) = o;
    }
}

// adjoint of upsample: coarse gradient (dense, C channels) = restriction of fine channels [fc0, fc0 + C)
__global__ void restrict_kernel(const float *__restrict__ fine, int fcs, int fc0, int hf, int wf,
                                float *__restrict__ coarse, int C, int hc, int wc, int batch) {
    const long long total = (long long)batch * hc * wc * C;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(idx % C);
        long long q = idx / C;
        const int X = (int)(q % wc);
        q /= wc;
        const int Y = (int)(q % hc);
        const int b = (int)(q / hc);
        float s = 0.0f;
        for (int dy = -1; dy <= 1; dy++) {
            const int y = 2 * Y + dy;
            if (y < 0 || y >= hf) continue;
            const float wy = dy == 0 ? 1.0f : 0.5f;
            for (int dx = -1; dx <= 1; dx++) {
                const int x = 2 * X + dx;
                if (x < 0 || x >= wf) continue;
                const float wx = dx == 0 ? 1.0f : 0.5f;
                s += wy * wx * fine[(((size_t)b * hf + y) * wf + x) * fcs + fc0 + c];
            }
        }
        coarse[idx] = s;
    }
}

// pre-activation gradient in bf16: gpre[p][c] = gpost[p][c] * (y[p][c] > 0), zero for c >= cout
__global__ void relu_grad_kernel(const float *__restrict__ gpost, int gcs, int gc0, const bf16 *__restrict__ y,
                                 int ycs, int yc0, int relu, int cout, int coutp, long long P,
                                 bf16 *__restrict__ gpre) {
    const long long total = P * coutp;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(idx % coutp);
        const long long p = idx / coutp;
        float g = 0.0f;
        if (c < cout) {
            g = gpost[p * gcs + gc0 + c];
            if (relu && !(__bfloat162float(y[p * ycs + yc0 + c]) > 0.0f)) g = 0.0f;
        }
        gpre[idx] = __float2bfloat16_rn(g);
    }
}

// weight gradient partials: part[z][co][tap][ci] = sum over this split's pixels of gpre[p][co] * x[src(p,tap)][ci]
__global__ void __launch_bounds__(128) dw_kernel(const __grid_constant__ DwArgs a) {
    __shared__ float Gs[32][33];
    __shared__ __align__(16) float Xs[32][9][34];
    const int tid = threadIdx.x, cg = tid >> 4, ig = tid & 15;
    const int co0 = blockIdx.x * 32, ci0 = blockIdx.y * 32;
    const long long P = (long long)a.batch * a.hout * a.wout;
    const long long pb = (long long)blockIdx.z * a.chunk;
    const long long pe = min(P, pb + a.chunk);
    float acc[9][4][2];
#pragma unroll
    for (int t = 0; t < 9; t++)
#pragma unroll
        for (int i = 0; i < 4; i++) acc[t][i][0] = acc[t][i][1] = 0.0f;
    for (long long p0 = pb; p0 < pe; p0 += 32) {
        {   // G rows: 32 pixels x 32 channels, 8 channels per thread
            const int pp = tid >> 2, cb = (tid & 3) * 8;
            const long long p = p0 + pp;
            float g[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (p < pe && co0 + cb < a.gc) {
                const uint4 u = *reinterpret_cast<const uint4 *>(a.g + p * a.gc + co0 + cb);
                const bf16 *h = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
                for (int j = 0; j < 8; j++) g[j] = __bfloat162float(h[j]);
            }
#pragma unroll
            for (int j = 0; j < 8; j++) Gs[pp][cb + j] = g[j];
        }
        for (int j = 0; j < 9; j++) {   // X at the 9 taps: 32 x 9 x 4 vectors of 8 channels
            const int idx = tid + 128 * j;
            const int pp = idx / 36, rem = idx % 36, tap = rem >> 2, cb = (rem & 3) * 8;
            const long long p = p0 + pp;
            float xv[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (p < pe && ci0 + cb < a.cin) {
                const int ox = (int)(p % a.wout);
                const long long q = p / a.wout;
                const int oy = (int)(q % a.hout), b = (int)(q / a.hout);
                int yi, xi;
                if (tap_src(a.stride == 1 ? kFwdS1 : kFwdS2, oy, ox, tap / 3 - 1, tap % 3 - 1, a.hin, a.win, yi,
                            xi)) {
                    const uint4 u = *reinterpret_cast<const uint4 *>(
                        a.x + (((size_t)b * a.hin + yi) * a.win + xi) * a.x_cs + a.x_c0 + ci0 + cb);
                    const bf16 *h = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
                    for (int e = 0; e < 8; e++) xv[e] = __bfloat162float(h[e]);
                }
            }
#pragma unroll
            for (int e = 0; e < 8; e++) Xs[pp][tap][cb + e] = xv[e];
        }
        __syncthreads();
        const int np = (int)min((long long)32, pe - p0);
        for (int pp = 0; pp < np; pp++) {
            float g[4];
#pragma unroll
            for (int i = 0; i < 4; i++) g[i] = Gs[pp][cg * 4 + i];
#pragma unroll
            for (int t = 0; t < 9; t++) {
                const float2 x2 = *reinterpret_cast<const float2 *>(&Xs[pp][t][ig * 2]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    acc[t][i][0] = fmaf(g[i], x2.x, acc[t][i][0]);
                    acc[t][i][1] = fmaf(g[i], x2.y, acc[t][i][1]);
                }
            }
        }
        __syncthreads();
    }
    float *dst = a.part + (size_t)blockIdx.z * a.cout * 9 * a.cin;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int co = co0 + cg * 4 + i;
        if (co >= a.cout) continue;
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int ci = ci0 + ig * 2 + j;
            if (ci >= a.cin) continue;
#pragma unroll
            for (int t = 0; t < 9; t++) dst[((size_t)co * 9 + t) * a.cin + ci] = acc[t][i][j];
        }
    }
}

// bias gradient partials: part[z][co] = sum over this split's pixels of gpre[p][co]
__global__ void bias_grad_kernel(const bf16 *__restrict__ g, int gc, int cout, long long P, long long chunk,
                                 float *__restrict__ part) {
    const int co = threadIdx.x;
    if (co >= cout) return;
    const long long pb = blockIdx.x * chunk, pe = min(P, pb + chunk);
    float s = 0.0f;
    for (long long p = pb; p < pe; p++) s += __bfloat162float(g[p * gc + co]);
    part[(size_t)blockIdx.x * cout + co] = s;
}

// out[i] = sum_z part[z][i] (fixed order)
__global__ void reduce_parts_kernel(const float *__restrict__ part, int nsplit, long long n, float *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int z = 0; z < nsplit; z++) s += part[(size_t)z * n + i];
        out[i] = s;
    }
}

// masked squared error: per-block partial sums of mask and of mask * (out - tgt)^2
constexpr int kLossBlocks = 256;
__global__ void loss_partial_kernel(const float *__restrict__ out, const float *__restrict__ tgt,
                                    const float *__restrict__ mask, long long n, double *__restrict__ part) {
    __shared__ double sm[96];
    double v[3] = {0.0, 0.0, 0.0};
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double m = mask ? (double)mask[i] : 1.0, d = (double)out[i] - (double)tgt[i];
        v[0] += m;
        v[1] += m * d * d;
        v[2] += m * (double)tgt[i] * (double)tgt[i];
    }
    block_sum<3>(v, sm);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 3] = v[0];
        part[blockIdx.x * 3 + 1] = v[1];
        part[blockIdx.x * 3 + 2] = v[2];
    }
}
// sums the partials (every block redundantly, fixed order) and writes the output gradient 2 m (o - t) / sum(m)
__global__ void loss_grad_kernel(const float *__restrict__ out, const float *__restrict__ tgt,
                                 const float *__restrict__ mask, long long n, const double *__restrict__ part,
                                 float *__restrict__ gout, double *__restrict__ loss, double *__restrict__ rel) {
    __shared__ double s_m;
    if (threadIdx.x == 0) {
        double m = 0.0, l = 0.0, t = 0.0;
        for (int b = 0; b < kLossBlocks; b++) {
            m += part[3 * b];
            l += part[3 * b + 1];
            t += part[3 * b + 2];
        }
        if (m <= 0.0) m = 1.0;
        s_m = m;
        if (blockIdx.x == 0 && loss) {
            loss[0] = l / m;
            if (rel) rel[0] = t > 0.0 ? l / t : 0.0;
        }
    }
    __syncthreads();
    const float sc = (float)(2.0 / s_m);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float m = mask ? mask[i] : 1.0f;
        gout[i] = sc * m * (out[i] - tgt[i]);
    }
}

__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float bc1,
                            float bc2) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

__global__ void f32_to_bf16_kernel(const float *__restrict__ in, long long n, bf16 *__restrict__ out) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(in[i]);
}

static int gsz(long long n, int block = 256) {
    long long g = (n + block - 1) / block;
    return (int)std::max(1ll, std::min(g, 152ll * 16));
}

// ------------------------------------------------------------------ host: the network object
Net::~Net() { release(); }

void Net::release() {
    for (void *p : allocs) cudaFree(p);
    allocs.clear();
}

template <typename T>
static psf_status net_alloc(Net *n, T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc (network)");
    n->allocs.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PSF_OK;
}

psf_status Net::init(int c0_, int H_, int W_, int batch_, uint64_t seed) {
    if (c0_ < 16 || c0_ % 16 != 0 || c0_ > 32) {
        set_error("network base width must be 16 or 32");
        return PSF_BAD_INPUT;
    }
    if (H_ < 9 || W_ < 9 || (H_ - 1) % 8 || (W_ - 1) % 8 || batch_ < 1) {
        set_error("network grid must be (8k+1) x (8m+1) nodes, at least 9 x 9, with batch >= 1");
        return PSF_BAD_INPUT;
    }
    PSF_CUDA(conv_init_attrs());
    c0 = c0_;
    H[0] = H_;
    W[0] = W_;
    cap = batch_;
    for (int l = 1; l < 4; l++) {
        H[l] = (H[l - 1] + 1) / 2;
        W[l] = (W[l - 1] + 1) / 2;
    }
    nparams = layer_table(c0, L);
    tensor_shape(c0, C, lev);
    PSF_CHECK(net_alloc(this, &params, nparams));
    PSF_CHECK(net_alloc(this, &grads, nparams));
    PSF_CHECK(net_alloc(this, &adam_m, nparams));
    PSF_CHECK(net_alloc(this, &adam_v, nparams));
    PSF_CUDA(cudaMemset(adam_m, 0, sizeof(float) * nparams));
    PSF_CUDA(cudaMemset(adam_v, 0, sizeof(float) * nparams));
    PSF_CHECK(net_alloc(this, &err, 4));
    PSF_CUDA(cudaMemset(err, 0, sizeof(int) * 4));
    PSF_CHECK(net_alloc(this, &dloss, 3 * kLossBlocks + 2));
    size_t part_max = 0;
    for (int l = 0; l < kLayers; l++) {
        const LayerDesc &y = L[l];
        const int coutp = pad16(y.cout);
        nchunk_f[l] = (9 * y.cin + 63) / 64;
        nchunk_b[l] = (9 * coutp + 63) / 64;
        PSF_CHECK(net_alloc(this, &wf[l], (size_t)nchunk_f[l] * 64 * coutp));
        wb[l] = nullptr;
        if (l > 0) PSF_CHECK(net_alloc(this, &wb[l], (size_t)nchunk_b[l] * 64 * y.cin));
        part_max = std::max(part_max, (size_t)kDwSplitMax * y.cout * 9 * y.cin + (size_t)kDwSplitMax * y.cout);
    }
    PSF_CHECK(net_alloc(this, &part, part_max));
    size_t gp_max = 0;
    for (int i = 0; i < kTensors; i++) {
        const size_t n = npix(lev[i]) * C[i];
        t[i] = nullptr;
        g[i] = nullptr;
        if (i < kTensors - 1) PSF_CHECK(net_alloc(this, &t[i], n));
        PSF_CHECK(net_alloc(this, &g[i], n));
        gp_max = std::max(gp_max, npix(lev[i]) * (size_t)pad16(C[i]));
    }
    PSF_CHECK(net_alloc(this, &out32, npix(0) * 2));
    PSF_CHECK(net_alloc(this, &gpre, gp_max));
    // He-normal initial weights, zero biases (host generator: splitmix64 + Box-Muller)
    std::vector<float> h(nparams, 0.0f);
    uint64_t st = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&st]() {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kLayers; l++) {
        const double sd = sqrt(2.0 / (9.0 * (l == 0 ? 7 : L[l].cin)));
        for (int i = L[l].woff; i < L[l].boff; i++) {
            const double u1 = next(), u2 = next();
            h[i] = (float)(sd * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
        }
        if (l == 0)  // the padded input channel 7 carries nothing
            for (int co = 0; co < L[0].cout; co++)
                for (int tp = 0; tp < 9; tp++) h[L[0].woff + ((size_t)co * 9 + tp) * 8 + 7] = 0.0f;
        if (l == kLayers - 1)
            for (int i = L[l].woff; i < L[l].boff; i++) h[i] *= 0.1f;
    }
    PSF_CUDA(cudaMemcpy(params, h.data(), sizeof(float) * nparams, cudaMemcpyHostToDevice));
    return pack();
}

psf_status Net::pack() {
    for (int l = 0; l < kLayers; l++) {
        const LayerDesc &y = L[l];
        const int coutp = pad16(y.cout);
        (pack_kernel<<<gsz((long long)nchunk_f[l] * 64 * coutp), 256, 0, stream>>>(
            params + y.woff, y.cout, y.cin, coutp, y.cin, nchunk_f[l], 0, wf[l]), ::psf::note_launch());
        if (wb[l])
            (pack_kernel<<<gsz((long long)nchunk_b[l] * 64 * y.cin), 256, 0, stream>>>(
                params + y.woff, y.cout, y.cin, y.cin, coutp, nchunk_b[l], 1, wb[l]), ::psf::note_launch());
    }
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status Net::forward(int B, const bf16 *input) {
    if (B < 1 || B > cap) {
        set_error("network batch exceeds its capacity");
        return PSF_BAD_INPUT;
    }
    const bf16 *tin[kTensors];
    for (int i = 0; i < kTensors; i++) tin[i] = t[i];
    tin[0] = input ? input : t[0];
    for (int l = 0; l < kLayers; l++) {
        const LayerDesc &y = L[l];
        if (l == 8 || l == 10 || l == 12) {
            const int src = l == 8 ? 8 : (l == 10 ? 10 : 12);
            const int dst = l == 8 ? 6 : (l == 10 ? 4 : 2);
            const int lc = lev[src], lf = lev[dst];
            const long long n = (long long)B * H[lf] * W[lf] * (C[src] / 8);
            (upsample_kernel<<<gsz(n), 256, 0, stream>>>(tin[src], C[src], H[lc], W[lc], t[dst], C[dst],
                                                        C[dst] - C[src], H[lf], W[lf], B, skip), ::psf::note_launch());
        }
        ConvArgs a{};
        a.x = tin[y.in];
        a.x_cs = y.in_cs;
        a.x_c0 = y.in_c0;
        a.cin = y.cin;
        a.hin = H[lev[y.in]];
        a.win = W[lev[y.in]];
        a.hout = H[y.level];
        a.wout = W[y.level];
        a.batch = B;
        a.w = wf[l];
        a.bias = params + y.boff;
        a.nchunks = nchunk_f[l];
        a.relu = y.relu;
        a.mode = y.stride == 1 ? kFwdS1 : kFwdS2;
        a.err = err;
        a.skip = skip;
        if (l == kLayers - 1) {
            a.y32 = out32;
            a.y_cs = 2;
            a.y_c0 = 0;
            a.cstore = 2;
        } else {
            a.y = t[y.out];
            a.y_cs = y.out_cs;
            a.y_c0 = y.out_c0;
            a.cstore = y.cout;
        }
        PSF_CUDA(launch_conv(pad16(y.cout), a, stream));
    }
    return PSF_OK;
}

psf_status Net::backward(int B, const bf16 *input) {
    const bf16 *tin[kTensors];
    for (int i = 0; i < kTensors; i++) tin[i] = t[i];
    tin[0] = input ? input : t[0];
    for (int l = kLayers - 1; l >= 0; l--) {
        const LayerDesc &y = L[l];
        const int coutp = pad16(y.cout);
        const long long Pout = (long long)B * H[y.level] * W[y.level];
        // pre-activation gradient (bf16, dense coutp channels)
        const bool last = l == kLayers - 1;
        (relu_grad_kernel<<<gsz(Pout * coutp), 256, 0, stream>>>(
            g[y.out], last ? 2 : y.out_cs, last ? 0 : y.out_c0, last ? nullptr : t[y.out], y.out_cs, y.out_c0,
            y.relu, y.cout, coutp, Pout, gpre), ::psf::note_launch());
        // weight and bias gradients
        const int tx = (y.cout + 31) / 32, ty = (y.cin + 31) / 32;
        int nsplit = (int)std::min<long long>(std::max(1, 608 / (tx * ty)), (Pout + 255) / 256);
        nsplit = std::max(1, std::min(nsplit, kDwSplitMax));
        DwArgs d{};
        d.g = gpre;
        d.gc = coutp;
        d.x = tin[y.in];
        d.x_cs = y.in_cs;
        d.x_c0 = y.in_c0;
        d.cin = y.cin;
        d.hin = H[lev[y.in]];
        d.win = W[lev[y.in]];
        d.hout = H[y.level];
        d.wout = W[y.level];
        d.batch = B;
        d.stride = y.stride;
        d.cout = y.cout;
        d.chunk = ((Pout + nsplit - 1) / nsplit + 31) / 32 * 32;
        nsplit = (int)((Pout + d.chunk - 1) / d.chunk);
        d.part = part;
        (dw_kernel<<<dim3(tx, ty, nsplit), 128, 0, stream>>>(d), ::psf::note_launch());
        const long long nw = (long long)y.cout * 9 * y.cin;
        (reduce_parts_kernel<<<gsz(nw), 256, 0, stream>>>(part, nsplit, nw, grads + y.woff), ::psf::note_launch());
        float *bpart = part + (size_t)kDwSplitMax * nw;
        (bias_grad_kernel<<<nsplit, 128, 0, stream>>>(gpre, coutp, y.cout, Pout, d.chunk, bpart), ::psf::note_launch());
        (reduce_parts_kernel<<<1, 128, 0, stream>>>(bpart, nsplit, y.cout, grads + y.boff), ::psf::note_launch());
        // data gradient into the input tensor's gradient (accumulating where a skip tensor has two consumers)
        if (l > 0) {
            ConvArgs a{};
            a.x = gpre;
            a.x_cs = coutp;
            a.x_c0 = 0;
            a.cin = coutp;
            a.hin = H[y.level];
            a.win = W[y.level];
            a.hout = H[lev[y.in]];
            a.wout = W[lev[y.in]];
            a.batch = B;
            a.w = wb[l];
            a.bias = nullptr;
            a.nchunks = nchunk_b[l];
            a.relu = 0;
            a.mode = y.stride == 1 ? kBwdS1 : kBwdS2;
            a.err = err;
            a.y32 = g[y.in];
            a.y_cs = y.in_cs;
            a.y_c0 = y.in_c0;
            a.cstore = y.cin;
            // layers 2, 4, 6 read the skip part of a concatenation whose gradient the decoder wrote first
            a.accumulate = (l == 2 || l == 4 || l == 6) ? 1 : 0;
            PSF_CUDA(launch_conv(y.cin, a, stream));
        }
        // gradient of an upsampled tensor: restriction of the concatenation's upper channels
        if (l == 12 || l == 10 || l == 8) {
            const int cat = l == 12 ? 2 : (l == 10 ? 4 : 6);
            const int src = l == 12 ? 12 : (l == 10 ? 10 : 8);
            const int lf = lev[cat], lc = lev[src];
            const long long n = (long long)B * H[lc] * W[lc] * C[src];
            (restrict_kernel<<<gsz(n), 256, 0, stream>>>(g[cat], C[cat], C[cat] - C[src], H[lf], W[lf], g[src],
                                                        C[src], H[lc], W[lc], B), ::psf::note_launch());
        }
    }
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status Net::loss_grad(int B, const float *tgt, const float *mask, double *d_loss, double *d_rel) {
    const long long n = npix_b(B, 0) * 2;
    (loss_partial_kernel<<<kLossBlocks, 256, 0, stream>>>(out32, tgt, mask, n, dloss), ::psf::note_launch());
    (loss_grad_kernel<<<gsz(n), 256, 0, stream>>>(out32, tgt, mask, n, dloss, g[kTensors - 1],
                                                  d_loss ? d_loss : dloss + 3 * kLossBlocks, d_rel),
                                                  ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return PSF_OK;
}

psf_status Net::adam(float lr) {
    step_count++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = 1.0f - powf(b1, (float)step_count), bc2 = 1.0f - powf(b2, (float)step_count);
    (adam_kernel<<<gsz(nparams), 256, 0, stream>>>(params, grads, adam_m, adam_v, nparams, lr, b1, b2, 1e-8f, bc1,
                                                  bc2), ::psf::note_launch());
    PSF_CUDA(cudaGetLastError());
    return pack();
}

psf_status Net::check_err() {
    int h = 0;
    PSF_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    PSF_CUDA(cudaStreamSynchronize(stream));
    if (h) {
        set_error("network convolution timed out waiting for the tensor cores");
        return PSF_TIMEOUT;
    }
    return PSF_OK;
}

psf_status Net::upload_input(int B, const float *host_in) {
    const long long n = npix_b(B, 0) * 8;
    float *tmp = nullptr;
    PSF_CUDA(cudaMalloc(&tmp, sizeof(float) * n));
    cudaError_t e = cudaMemcpyAsync(tmp, host_in, sizeof(float) * n, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) {
        (f32_to_bf16_kernel<<<gsz(n), 256, 0, stream>>>(tmp, n, t[0]), ::psf::note_launch());
        e = cudaStreamSynchronize(stream);
    }
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_status(e, "network input upload");
    return PSF_OK;
}

}  // namespace unet
}  // namespace psf

// ------------------------------------------------------------------ C ABI
using psf::unet::bf16;
using psf::unet::ConvArgs;
using psf::unet::f32_to_bf16_kernel;
using psf::unet::gsz;
using psf::unet::launch_conv;
using psf::unet::pack_kernel;

extern "C" {

psf_status psf_unet_create(int c0, int H, int W, int batch, uint64_t seed, psf_unet **out) {
    if (!out) return PSF_BAD_INPUT;
    *out = nullptr;
    psf_unet *u = new psf_unet();
    using psf::unet::Net;
    psf_status s = u->net.init(c0, H, W, batch, seed);
    if (s == PSF_OK) s = psf::cuda_status(cudaStreamSynchronize(u->net.stream), "network init");
    if (s != PSF_OK) {
        delete u;
        return s;
    }
    *out = u;
    return PSF_OK;
}

psf_status psf_unet_destroy(psf_unet *u) {
    delete u;
    return PSF_OK;
}

int psf_unet_nparams(const psf_unet *u) { return u ? u->net.nparams : 0; }

psf_status psf_unet_set_params(psf_unet *u, const float *host, int n) {
    if (!u || !host || n != u->net.nparams) {
        psf::set_error("psf_unet_set_params: parameter count mismatch");
        return PSF_BAD_INPUT;
    }
    PSF_CUDA(cudaMemcpy(u->net.params, host, sizeof(float) * n, cudaMemcpyHostToDevice));
    PSF_CHECK(u->net.pack());
    PSF_CUDA(cudaStreamSynchronize(u->net.stream));
    return PSF_OK;
}

psf_status psf_unet_get_params(const psf_unet *u, float *host, int n) {
    if (!u || !host || n != u->net.nparams) {
        psf::set_error("psf_unet_get_params: parameter count mismatch");
        return PSF_BAD_INPUT;
    }
    PSF_CUDA(cudaMemcpy(host, u->net.params, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return PSF_OK;
}

psf_status psf_unet_get_out_scale(const psf_unet *u, float *scale) {
    if (!u || !scale) return PSF_BAD_INPUT;
    *scale = u->net.out_scale;
    return PSF_OK;
}

psf_status psf_unet_set_out_scale(psf_unet *u, float scale) {
    if (!u || !(scale > 0.0f)) return PSF_BAD_INPUT;
    u->net.out_scale = scale;
    return PSF_OK;
}

psf_status psf_unet_forward_host(psf_unet *u, int B, const float *in, float *out) {
    if (!u || !in || !out) return PSF_BAD_INPUT;
    psf::unet::Net &n = u->net;
    if (B < 1 || B > n.cap) return PSF_BAD_INPUT;
    PSF_CHECK(n.upload_input(B, in));
    PSF_CHECK(n.forward(B, nullptr));
    PSF_CHECK(n.check_err());
    PSF_CUDA(cudaMemcpy(out, n.out32, sizeof(float) * n.npix_b(B, 0) * 2, cudaMemcpyDeviceToHost));
    return PSF_OK;
}

psf_status psf_unet_loss_grad_host(psf_unet *u, int B, const float *in, const float *tgt, const float *mask,
                                   double *loss, float *out, float *grad) {
    if (!u || !in || !tgt) return PSF_BAD_INPUT;
    psf::unet::Net &n = u->net;
    if (B < 1 || B > n.cap) return PSF_BAD_INPUT;
    const size_t no = n.npix_b(B, 0) * 2;
    float *dt = nullptr, *dm = nullptr;
    double *dl = nullptr;
    PSF_CUDA(cudaMalloc(&dt, sizeof(float) * no * 2));
    dm = dt + no;
    PSF_CUDA(cudaMalloc(&dl, sizeof(double)));
    psf_status s = n.upload_input(B, in);
    if (s == PSF_OK) s = psf::cuda_status(cudaMemcpy(dt, tgt, sizeof(float) * no, cudaMemcpyHostToDevice), "copy");
    if (s == PSF_OK && mask)
        s = psf::cuda_status(cudaMemcpy(dm, mask, sizeof(float) * no, cudaMemcpyHostToDevice), "copy");
    if (s == PSF_OK) s = n.forward(B, nullptr);
    if (s == PSF_OK) s = n.loss_grad(B, dt, mask ? dm : nullptr, dl, nullptr);
    if (s == PSF_OK) s = n.backward(B, nullptr);
    if (s == PSF_OK) s = n.check_err();
    if (s == PSF_OK && loss) s = psf::cuda_status(cudaMemcpy(loss, dl, sizeof(double), cudaMemcpyDeviceToHost), "copy");
    if (s == PSF_OK && out)
        s = psf::cuda_status(cudaMemcpy(out, n.out32, sizeof(float) * no, cudaMemcpyDeviceToHost), "copy");
    if (s == PSF_OK && grad)
        s = psf::cuda_status(cudaMemcpy(grad, n.grads, sizeof(float) * n.nparams, cudaMemcpyDeviceToHost), "copy");
    cudaFree(dt);
    cudaFree(dl);
    return s;
}

psf_status psf_unet_conv(int mode, int N, int cin, int hin, int win, int hout, int wout, int B, const float *x,
                         const float *w, const float *bias, int relu, float *y) {
    using namespace psf::unet;
    if (mode < 0 || mode > 3 || cin < 8 || cin % 8 || B < 1 || hin < 1 || win < 1 || hout < 1 || wout < 1 || !x ||
        !w || !y) {
        psf::set_error("psf_unet_conv: bad arguments");
        return PSF_BAD_INPUT;
    }
    if (N != 16 && N != 32 && N != 48 && N != 64 && N != 96 && N != 128 && N != 192) {
        psf::set_error("psf_unet_conv: N must be one of 16, 32, 48, 64, 96, 128, 192");
        return PSF_BAD_INPUT;
    }
    const size_t nx = (size_t)B * hin * win * cin, nw = (size_t)N * 9 * cin, ny = (size_t)B * hout * wout * N;
    const int nchunks = (9 * cin + 63) / 64;
    float *fx = nullptr, *fw = nullptr, *fb = nullptr, *fy = nullptr;
    bf16 *bx = nullptr, *bw = nullptr;
    int *err = nullptr;
    psf_status s = PSF_OK;
    auto ck = [&s](cudaError_t e) {
        if (s == PSF_OK && e != cudaSuccess) s = psf::cuda_status(e, "psf_unet_conv");
    };
    ck(cudaMalloc(&fx, nx * 4));
    ck(cudaMalloc(&fw, nw * 4));
    ck(cudaMalloc(&fb, N * 4));
    ck(cudaMalloc(&fy, ny * 4));
    ck(cudaMalloc(&bx, nx * 2));
    ck(cudaMalloc(&bw, (size_t)nchunks * 64 * N * 2));
    ck(cudaMalloc(&err, 4));
    if (s == PSF_OK) {
        ck(cudaMemcpy(fx, x, nx * 4, cudaMemcpyHostToDevice));
        ck(cudaMemcpy(fw, w, nw * 4, cudaMemcpyHostToDevice));
        ck(cudaMemset(fb, 0, N * 4));
        if (bias) ck(cudaMemcpy(fb, bias, N * 4, cudaMemcpyHostToDevice));
        ck(cudaMemset(err, 0, 4));
    }
    if (s == PSF_OK) {
        (f32_to_bf16_kernel<<<gsz((long long)nx), 256>>>(fx, (long long)nx, bx), ::psf::note_launch());
        (pack_kernel<<<gsz((long long)nchunks * 64 * N), 256>>>(
             fw, N, cin, N, cin, nchunks, 0, bw),
         ::psf::note_launch());
        ConvArgs a{};
        a.x = bx;
        a.x_cs = cin;
        a.cin = cin;
        a.hin = hin;
        a.win = win;
        a.y32 = fy;
        a.y_cs = N;
        a.cstore = N;
        a.hout = hout;
        a.wout = wout;
        a.batch = B;
        a.w = bw;
        a.bias = fb;
        a.nchunks = nchunks;
        a.relu = relu;
        a.mode = mode;
        a.err = err;
        ck(launch_conv(N, a, 0));
        ck(cudaDeviceSynchronize());
        int h = 0;
        ck(cudaMemcpy(&h, err, 4, cudaMemcpyDeviceToHost));
        if (s == PSF_OK && h) {
            psf::set_error("psf_unet_conv: tensor-core wait timed out");
            s = PSF_TIMEOUT;
        }
        if (s == PSF_OK) ck(cudaMemcpy(y, fy, ny * 4, cudaMemcpyDeviceToHost));
    }
    cudaFree(fx);
    cudaFree(fw);
    cudaFree(fb);
    cudaFree(fy);
    cudaFree(bx);
    cudaFree(bw);
    cudaFree(err);
    return s;
}

}  // extern "C"
