// qs_resident.cu -- the slice loop of 256 x 256 waves with each wave resident
// on chip for all of its slices.
//
// One cluster of four CTAs (one per SM) carries one wave through every step
// of runMulsSTEM's loop (stem3/stemlib.cpp:2403-2486: transmit, FFT2,
// propagate_slow, collectIntensity, IFFT2, 1/N).  The wave never goes back to
// HBM between slices: between the transforms along y and along x it is
// redistributed across the cluster through distributed shared memory.
//
//   row layout     CTA r keeps rows x in [64r, 64r + 64), each as a padded
//                  line of 271 float2 (element y at y + y/16, the row
//                  transform's exchange layout), in-band columns only
//   column layout  CTA r keeps band columns j in [44r, 44r + 44) (the
//                  columns the 2/3 band limit keeps, numbered in order), all
//                  256 x, element x of column c at x*44 + c
//
// Per step:
//   row phase     (all 1024 threads: 64 lines of 16) IFFT_y of the row (the
//                 first step reads the incident wave instead), 1/N, transmit
//                 with the step's slice, FFT_y; each in-band value goes to
//                 the column layout of the CTA that owns its column
//   cluster barrier
//   column phase  (704 threads: 44 lines of 16) FFT_x, propagator and band
//                 limit, detector sums and the pattern on output steps,
//                 IFFT_x; each value goes back to the row layout of the CTA
//                 that owns its row
//   cluster barrier
// Each layout is also the exchange scratch of the transforms that read it,
// so the CTA holds 64*271 + 256*44 float2 plus the twiddles: 231 KB.
//
// Every CTA of a cluster runs the same number of cluster barriers (the step
// count is a kernel argument), so no barrier waits on a CTA that has left;
// every remote access happens between the first and the last of them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <string>

#include "qs_fft.cuh"
#include "qs_internal.h"

namespace qs {
namespace cg = cooperative_groups;

namespace {
constexpr int RN = 256;                // line length (nx = ny)
constexpr int RCL = 4;                 // CTAs per cluster (one wave)
constexpr int RROWS = RN / RCL;        // rows per CTA
constexpr int RSTRIDE = 271;           // padded row: y + y/16 for y < 256
constexpr int RCP = 44;                // band columns per CTA
constexpr int RTHREADS = 1024;         // 64 row lines of 16 threads
constexpr int RCOLT = 16 * RCP;        // 704 threads: 44 column lines of 16
using RCfg = Line<RN>::cfg;
static_assert(std::is_same<RCfg, LineCol<RN>::cfg>::value, "rows and columns share one transform");
static_assert(RCfg::T == 16 && RCfg::E == 16 && RCfg::R0 == 16, "row lines of 16 threads, first radix 16");
static_assert(RTHREADS == RROWS * RCfg::T, "one row line per 16 threads");
constexpr size_t RSMEM = sizeof(float2) * ((size_t)RROWS * RSTRIDE + (size_t)RN * RCP + RCfg::TW);
using ColBar = NamedBarrier<1, RCOLT>;

// 32-bit shared-window address of a pointer into this CTA's shared memory
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// the same offset in the shared memory of CTA `rank` of the cluster
__device__ __forceinline__ uint32_t cluster_addr(uint32_t a, int rank) {
    uint32_t r;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void st_cluster(uint32_t addr, float2 v) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(addr), "f"(v.x), "f"(v.y) : "memory");
}
}  // namespace

__global__ void __cluster_dims__(RCL, 1, 1) __launch_bounds__(RTHREADS, 1) ms_resident256(ResidentArgs a) {
    constexpr int T = RCfg::T, E = RCfg::E;
    extern __shared__ float2 dsm[];
    float2* s_rows = dsm;
    float2* s_cols = s_rows + RROWS * RSTRIDE;
    float2* s_tw = s_cols + RN * RCP;
    __shared__ double s_det[QS_MAX_DETECTORS];

    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int b = (int)(blockIdx.x / RCL);  // the cluster's wave
    const int tid = threadIdx.x;
    for (int i = tid; i < RCfg::TW; i += RTHREADS) s_tw[i] = a.tw[i];
    if (tid < QS_MAX_DETECTORS) s_det[tid] = 0.0;
    const uint32_t rows_u32 = smem_u32(s_rows), cols_u32 = smem_u32(s_cols);
    __syncthreads();
    cl.sync();  // every CTA of the cluster runs before the first remote store

    const int na = a.yA + 1 < RN ? a.yA + 1 : RN;  // band columns 0..na-1 are ky = j
    // row phase: line `line` of this CTA is row x, thread t holds y = t + 16e
    const int line = tid >> 4, t = tid & 15;
    const int x = rank * RROWS + line;
    float2* myrow = s_rows + line * RSTRIDE;
    const SmemRow<RCfg::R0> smr{myrow};
    // column phase: thread (c, ct) of band column j holds x = ct + 16e
    const bool colThread = tid < RCOLT;
    const int c = tid % RCP, ct = tid / RCP;
    const int j = rank * RCP + c;
    const bool colValid = colThread && j < a.nb;
    const int ky = j < na ? j : a.yB + (j - na);
    const int pX = __ldg(a.posX + b), pY = __ldg(a.posY + b);
    const size_t N2 = (size_t)RN * RN;
    const float2* stack = a.trans + (size_t)b * a.trans_stride;

    for (int step = 0; step < a.nsteps; ++step) {
        // ------------------------------------------------------ row phase
        float2 reg[E];
        if (step == 0) {
            const float2* src = a.probe + (size_t)b * a.probe_stride + (size_t)x * RN;
#pragma unroll
            for (int e = 0; e < E; ++e) reg[e] = __ldg(src + t + T * e);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int y = t + T * e;
                reg[e] = (!always_out_of_band<RN, T>(e) && (y <= a.yA || y >= a.yB)) ? smr(y)
                                                                                     : make_float2(0.f, 0.f);
            }
            line_fft<RCfg, true>(reg, smr, s_tw, t);
#pragma unroll
            for (int e = 0; e < E; ++e) reg[e] = cscale(reg[e], a.norm);
        }
        {
            // transmit (stem3/stemlib.cpp:2867-2888): window at (posX, posY)
            const float2* tr = stack + (size_t)__ldg(a.step_slice + step) * a.potNx * a.potNy +
                               (size_t)(x + pX) * a.potNy + pY;
#pragma unroll
            for (int e = 0; e < E; ++e) reg[e] = cmul(reg[e], __ldg(tr + t + T * e));
        }
        line_fft<RCfg, false>(reg, smr, s_tw, t);
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            if (always_out_of_band<RN, T>(e) || !(y <= a.yA || y >= a.yB)) continue;
            const int jj = y < na ? y : na + (y - a.yB);
            const int q = jj / RCP;
            st_cluster(cluster_addr(cols_u32 + (uint32_t)sizeof(float2) * (x * RCP + (jj - q * RCP)), q), reg[e]);
        }
        cl.sync();

        // --------------------------------------------------- column phase
        const int slot = __ldg(a.step_slot + step);
        const bool last = step == a.nsteps - 1;
        if (colThread) {
            float2 creg[E];
#pragma unroll
            for (int e = 0; e < E; ++e)
                creg[e] = colValid ? s_cols[(ct + T * e) * RCP + c] : make_float2(0.f, 0.f);
            ColBar::sync();  // all elements read before the layout becomes exchange scratch
            const SmemCol<RCP> smc{s_cols, c};
            line_fft_sync<RCfg, false, ColBar>(creg, smc, s_tw, ct);
            // propagate_slow (stem3/stemlib.cpp:2831-2849)
            const float ky2 = colValid ? __ldg(a.ky2 + ky) : a.k2max;
            const float2 pyv = colValid ? __ldg(a.py + ky) : make_float2(0.f, 0.f);
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int kx = ct + T * e;
                const float kx2 = __ldg(a.kx2 + kx);
                if (!always_out_of_band<RN, T>(e) && kx2 < a.k2max && (kx2 + ky2) < a.k2max)
                    creg[e] = cmul(cmul(creg[e], pyv), __ldg(a.px + kx));
                else
                    creg[e] = make_float2(0.f, 0.f);
            }
            if (slot >= 0 && a.ndet > 0) {
                // collectIntensity (stem3/stemlib.cpp:2615-2657): per thread
                // and warp in float, across warps and CTAs in double
                const int lane = tid & 31;
                for (int d = 0; d < a.ndet; ++d) {
                    float acc = 0.f;
                    const float lo = a.k2in[d], hi = a.k2out[d];
#pragma unroll
                    for (int e = 0; e < E; ++e) {
                        const float k2 = __ldg(a.kx2 + ct + T * e) + ky2;
                        const float I = creg[e].x * creg[e].x + creg[e].y * creg[e].y;
                        if (k2 >= lo && k2 <= hi) acc += I;
                    }
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                    if (lane == 0) atomicAdd(&s_det[d], (double)acc);
                }
                ColBar::sync();
                if (tid < a.ndet) {
                    a.partial[(size_t)slot * a.partial_slot + ((size_t)b * RCL + rank) * a.ndet + tid] = s_det[tid];
                    s_det[tid] = 0.0;
                }
            }
            float* dp = a.series ? (slot >= 0 ? a.diffpat + (size_t)slot * a.dp_slot : nullptr)
                                 : (last ? a.diffpat : nullptr);
            if (dp && colValid) {
                dp += (size_t)b * N2 + (ky + RN / 2) % RN;
                const float sc = (float)a.scaleDiff;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int kx = ct + T * e;
                    const float I = creg[e].x * creg[e].x + creg[e].y * creg[e].y;
                    dp[(size_t)((kx + RN / 2) % RN) * RN] = I * sc;
                }
            }
            if (!last || a.exit_waves) {
                // (the forward transform's last exchange ended with a barrier
                // after every read of the scratch)
                line_fft_sync<RCfg, true, ColBar>(creg, smc, s_tw, ct);
                if (colValid) {
                    const uint32_t off = rows_u32 + (uint32_t)sizeof(float2) * (ct * RSTRIDE + ky + ky / RCfg::R0);
#pragma unroll
                    for (int e = 0; e < E; ++e)
                        st_cluster(cluster_addr(off + (uint32_t)sizeof(float2) * (T * (e % 4) * RSTRIDE), e / 4),
                                   creg[e]);
                }
            }
        }
        cl.sync();
    }

    if (a.exit_waves) {
        // the real-space wave after the last step: IFFT_y, 1/N
        float2 reg[E];
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int y = t + T * e;
            reg[e] = (!always_out_of_band<RN, T>(e) && (y <= a.yA || y >= a.yB)) ? smr(y) : make_float2(0.f, 0.f);
        }
        line_fft<RCfg, true>(reg, smr, s_tw, t);
        float2* dst = a.exit_waves + (size_t)b * N2 + (size_t)x * RN;
#pragma unroll
        for (int e = 0; e < E; ++e) dst[t + T * e] = cscale(reg[e], a.norm);
    }
}

// Clusters of ms_resident256 that fit on the device at once (0: none; the
// caller then takes the two-pass loop).
int resident_clusters(int* out) {
    *out = 0;
    QS_TRY(smem_attr((const void*)ms_resident256, RSMEM));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(RCL, 1, 1);
    cfg.blockDim = dim3(RTHREADS, 1, 1);
    cfg.dynamicSmemBytes = RSMEM;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (const void*)ms_resident256, &cfg) != cudaSuccess) {
        (void)cudaGetLastError();
        return QS_OK;
    }
    *out = n;
    return QS_OK;
}

int resident_band_columns() { return RCL * RCP; }

int launch_resident(const ResidentArgs& a, cudaStream_t s) {
    if (a.nwaves < 1 || a.nsteps < 1) return QS_OK;
    if (a.nb < 0 || a.nb > RCL * RCP || a.ndet > QS_MAX_DETECTORS) {
        set_error("resident slice loop: band or detector count out of range");
        return QS_ERR_ARG;
    }
    QS_TRY(smem_attr((const void*)ms_resident256, RSMEM));
    ms_resident256<<<(unsigned)(a.nwaves * RCL), RTHREADS, RSMEM, s>>>(a);
    QS_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return QS_OK;
}

}  // namespace qs
