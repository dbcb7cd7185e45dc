// qs_noalloc.cu -- qs_multislice_run_noalloc: the multislice scan without any
// device allocation.
//
// Who needs this: callers that must not call cudaMalloc/cudaFree from inside
// their processing loop.  cudaFree waits for the whole device, so one call
// stalls every other stream of a process that shares the GPU; frameworks whose
// caching allocator owns the device memory see raw allocations as foreign
// memory they cannot reuse or account for; and deployments that reserve their
// full memory budget at start-up may have nothing left to allocate later.
// For them this entry point works entirely inside one fixed scratch area that
// lives in the library image itself, plus the buffers the caller passes.
//
// The scratch is a file-scope __device__ array of QS_NOALLOC_SCRATCH_BYTES.
// Every GPU that loads the library holds it until the process exits.  Host
// code cannot use the array's name as a device address, so the first call on
// each device looks the address up with cudaGetSymbolAddress (with that
// device current) and keeps it; make that first call before any stream
// capture.  All calls on a device share the one array and it keeps the
// previous call's contents: calls whose GPU work overlaps (different streams,
// or different host threads) race on it and must be serialised by the caller.
// The stream must belong to the device that is current when the call is made
// (that device's copy of the array is the one the kernels are given).
//
// The call's small tables (twiddles, propagator, k^2, column tiles, window
// offsets) reach the scratch as kernel arguments of a store kernel, so the
// work it queues refers to no host memory once it has returned.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "qs_fft.cuh"
#include "qs_internal.h"

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[QS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int scratch_address(void** out) {
    int dev = 0;
    QS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        qs::set_error("qs_multislice_run_noalloc: device ordinal out of range");
        return QS_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            qs::set_error(std::string("qs_multislice_run_noalloc: cudaGetSymbolAddress failed: ") +
                          cudaGetErrorString(e));
            return QS_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return QS_OK;
}

// Bump allocator over the scratch area (256-byte aligned pieces).
struct Carve {
    unsigned char* base;
    size_t used = 0;
    void* take(size_t bytes) {
        void* p = base + used;
        used += (bytes + 255) & ~(size_t)255;
        return p;
    }
};

// Host values carried to the scratch inside a kernel's parameter block
// (under the 4 KB parameter limit of every launch form), one launch per
// chunk: the launch copies the values when it is queued.
constexpr int kBlobWords = 960;
struct Blob {
    unsigned n;
    unsigned w[kBlobWords];
};

__global__ void blob_store(unsigned* __restrict__ dst, Blob b) {
    for (unsigned i = threadIdx.x; i < b.n; i += blockDim.x) dst[i] = b.w[i];
}

// Store `bytes` (a multiple of 4) of host data at device address dst.
int upload(void* dst, const void* src, size_t bytes, cudaStream_t s) {
    const unsigned char* q = (const unsigned char*)src;
    unsigned* d = (unsigned*)dst;
    for (size_t off = 0; off < bytes; off += sizeof(unsigned) * kBlobWords) {
        Blob b;
        const size_t chunk = std::min(bytes - off, sizeof(unsigned) * kBlobWords);
        b.n = (unsigned)(chunk / sizeof(unsigned));
        std::memcpy(b.w, q + off, chunk);
        blob_store<<<1, 256, 0, s>>>(d + off / sizeof(unsigned), b);
        QS_CUDA_TRY(cudaGetLastError());
        qs::count_launch(1);
    }
    return QS_OK;
}

}  // namespace

using namespace qs;

extern "C" int qs_multislice_run_noalloc(void* stream_handle, const qs_params* p, const float* trans_in,
                                         const float* probe_in, const qs_batch* batch, float* det_images,
                                         float* diffpats, float* exit_waves) {
    const char* fn = "qs_multislice_run_noalloc: ";
    if (!p || !trans_in || !probe_in || !batch) {
        set_error(std::string(fn) + "params, trans, probe and batch are required");
        return QS_ERR_ARG;
    }
    QS_TRY(check_params(p));
    const qs_params& P = *p;
    if (P.cellDiv != 1 || P.mulsRepeat1 > 1 || P.mulsRepeat2 > 1) {
        set_error(std::string(fn) + "slabs (cellDiv > 1) and stacking sequences other than 1 1 are not supported");
        return QS_ERR_ARG;
    }
    if (!line_supported(P.nx) || !line_supported(P.ny)) {
        set_error(std::string(fn) + "nx, ny must be in {64,128,256,384,512,768,1024}");
        return QS_ERR_UNSUPPORTED;
    }
    for (int d = 0; d < P.detectorNum; d++)
        if (P.detectors[d].shiftX != 0 || P.detectors[d].shiftY != 0) {
            set_error(std::string(fn) + "shifted detectors are not supported");
            return QS_ERR_UNSUPPORTED;
        }
    const int npos = batch->npos;
    if (npos < 1) {
        set_error(std::string(fn) + "batch has no positions");
        return QS_ERR_ARG;
    }
    const int nx = P.nx, ny = P.ny, S = P.slices;
    const size_t N = (size_t)nx * ny;
    const int nT = (P.slices * P.cellDiv) / P.outputInterval + 1;
    const int ndet = P.detectorNum;
    const int npix = P.scanXN * P.scanYN;
    const bool wantDet = ndet > 0 && det_images != nullptr;
    QS_TRY(check_raster(P, *batch, wantDet));
    cudaStream_t s = (cudaStream_t)stream_handle;
    {
        // the scratch address handed to the kernels is the current device's;
        // the stream's device cannot be queried while the stream captures
        // (the capture's launches then fail if the two differ)
        int cur = 0, sdev = 0;
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        QS_CUDA_TRY(cudaGetDevice(&cur));
        QS_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
        if (cap == cudaStreamCaptureStatusNone) QS_CUDA_TRY(cudaStreamGetDevice(s, &sdev));
        else sdev = cur;
        if (sdev != cur) {
            set_error(std::string(fn) + "the stream belongs to device " + std::to_string(sdev) +
                      ", the current device is " + std::to_string(cur));
            return QS_ERR_ARG;
        }
    }

    // positions, as doSTEM computes them when the batch gives none
    std::vector<int> pos(4 * (size_t)npos);
    int *px_ = pos.data(), *py_ = px_ + npos, *dx_ = py_ + npos, *dy_ = dx_ + npos;
    for (int i = 0; i < npos; i++) {
        if (batch->iPosX && batch->iPosY) {
            px_[i] = batch->iPosX[i];
            py_[i] = batch->iPosY[i];
        } else {
            const int ix = i / P.scanYN, iy = i % P.scanYN;
            int x = (int)((float)ix * (P.scanXStop - P.scanXStart) / ((float)P.scanXN * P.resolutionX));
            int y = (int)((float)iy * (P.scanYStop - P.scanYStart) / ((float)P.scanYN * P.resolutionY));
            px_[i] = std::min(x, P.potNx - nx);
            py_[i] = std::min(y, P.potNy - ny);
        }
        // raster pixels (check_raster: scanYN >= 1 whenever they are used)
        dx_[i] = batch->detPosX ? batch->detPosX[i] : (P.scanYN > 0 ? i / P.scanYN : 0);
        dy_[i] = batch->detPosY ? batch->detPosY[i] : (P.scanYN > 0 ? i % P.scanYN : 0);
        if (px_[i] < 0 || py_[i] < 0 || px_[i] > P.potNx - nx || py_[i] > P.potNy - ny) {
            set_error(std::string(fn) + "position " + std::to_string(i) + " puts the window outside the potential");
            return QS_ERR_ARG;
        }
        if (wantDet && (dx_[i] < 0 || dx_[i] >= P.scanXN || dy_[i] < 0 || dy_[i] >= P.scanYN)) {
            set_error(std::string(fn) + "detector pixel of position " + std::to_string(i) + " outside the raster");
            return QS_ERR_ARG;
        }
    }

    // propagator tables, band and column tiles (the same as qs_multislice_run's)
    const PropTables tb = prop_tables(P);
    const Band band = band_tiles(tb, ny, col_tile_width(nx));
    const int ntiles = (int)band.tiles.size();
    std::vector<int> lastWriter(nT, -1), slotOf(S, -1);
    for (int sl = 0; sl < S; sl++) lastWriter[(sl < S * P.cellDiv - 1) ? sl / P.outputInterval : nT - 1] = sl;
    for (int t = 0; t < nT; t++) if (lastWriter[t] >= 0) slotOf[lastWriter[t]] = t;

    // scratch layout; the whole batch must fit
    const size_t partPerT = (size_t)npos * ntiles * std::max(ndet, 1);
    auto rup = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t need = rup(sizeof(float2) * ny) + rup(sizeof(float2) * nx) + rup(sizeof(float) * nx) +
                        rup(sizeof(float) * ny) + rup(sizeof(float2) * nx) + rup(sizeof(float2) * ny) +
                        rup(sizeof(int) * std::max(ntiles, 1)) + rup(sizeof(int) * 4 * (size_t)npos) +
                        rup(sizeof(double) * partPerT * nT) + rup(sizeof(float2) * N * npos);
    if (need > (size_t)QS_NOALLOC_SCRATCH_BYTES) {
        set_error(std::string(fn) + "this batch needs " + std::to_string(need) + " bytes of scratch; the fixed area holds " +
                  std::to_string((size_t)QS_NOALLOC_SCRATCH_BYTES) + " (split the positions into smaller batches)");
        return QS_ERR_ARG;
    }
    void* base = nullptr;
    QS_TRY(scratch_address(&base));
    Carve cv{(unsigned char*)base};
    float2* d_tw_y = (float2*)cv.take(sizeof(float2) * ny);
    float2* d_tw_x = (float2*)cv.take(sizeof(float2) * nx);
    float* d_kx2 = (float*)cv.take(sizeof(float) * nx);
    float* d_ky2 = (float*)cv.take(sizeof(float) * ny);
    float2* d_px = (float2*)cv.take(sizeof(float2) * nx);
    float2* d_py = (float2*)cv.take(sizeof(float2) * ny);
    int* d_tiles = (int*)cv.take(sizeof(int) * std::max(ntiles, 1));
    int* d_pos = (int*)cv.take(sizeof(int) * 4 * (size_t)npos);
    double* d_part = (double*)cv.take(sizeof(double) * partPerT * nT);
    float2* waves = (float2*)cv.take(sizeof(float2) * N * npos);

    std::vector<float2> twy, twx;
    QS_TRY(twiddle_host(ny, twy));
    QS_TRY(twiddle_host(nx, twx, true));
    QS_TRY(upload(d_tw_y, twy.data(), sizeof(float2) * ny, s));
    QS_TRY(upload(d_tw_x, twx.data(), sizeof(float2) * nx, s));
    QS_TRY(upload(d_kx2, tb.kx2.data(), sizeof(float) * nx, s));
    QS_TRY(upload(d_ky2, tb.ky2.data(), sizeof(float) * ny, s));
    QS_TRY(upload(d_px, tb.px.data(), sizeof(float2) * nx, s));
    QS_TRY(upload(d_py, tb.py.data(), sizeof(float2) * ny, s));
    if (ntiles) QS_TRY(upload(d_tiles, band.tiles.data(), sizeof(int) * ntiles, s));
    QS_TRY(upload(d_pos, pos.data(), sizeof(int) * 4 * (size_t)npos, s));
    // the previous call's waves are still in the area: clear them, and the
    // caller's outputs that are only partly written
    QS_CUDA_TRY(cudaMemsetAsync(waves, 0, sizeof(float2) * N * npos, s));
    if (wantDet) QS_CUDA_TRY(cudaMemsetAsync(det_images, 0, sizeof(float) * (size_t)nT * ndet * npix, s));
    if (diffpats) QS_CUDA_TRY(cudaMemsetAsync(diffpats, 0, sizeof(float) * N * npos, s));

    RowArgs ra{};
    ra.nx = nx; ra.ny = ny; ra.potNx = P.potNx; ra.potNy = P.potNy; ra.nwaves = npos;
    ra.probe = (const float2*)probe_in; ra.waves = waves; ra.exit_waves = (float2*)exit_waves;
    ra.posX = d_pos; ra.posY = d_pos + npos; ra.tw = d_tw_y; ra.yA = band.yA; ra.yB = band.yB;
    ra.norm = (float)(1.0 / (double)(nx * ny));
    ColArgs ca{};
    ca.nx = nx; ca.ny = ny; ca.nwaves = npos; ca.waves = waves; ca.tw = d_tw_x;
    ca.kx2 = d_kx2; ca.ky2 = d_ky2; ca.px = d_px; ca.py = d_py; ca.k2max = tb.k2max;
    ca.tiles = d_tiles; ca.ntiles = ntiles;
    for (int d = 0; d < ndet; d++) {
        ca.k2in[d] = P.detectors[d].k2Inside;
        ca.k2out[d] = P.detectors[d].k2Outside;
    }
    ca.scaleDiff = 1.0 / std::sqrt((double)(nx * ny));
    const float2* trans = (const float2*)trans_in;
    ra.trans_slice = trans;
    QS_TRY(launch_rows(ra, ROW_FIRST, s));
    for (int sl = 0; sl < S; sl++) {
        const int slot = slotOf[sl];
        ca.ndet = (wantDet && slot >= 0) ? ndet : 0;
        ca.partial = d_part + (slot >= 0 ? (size_t)slot * partPerT : 0);
        ca.diffpat = (sl == S - 1) ? diffpats : nullptr;
        ca.inverse = (sl < S - 1 || exit_waves) ? 1 : 0;
        QS_TRY(launch_cols(ca, s));
        if (sl < S - 1) {
            ra.trans_slice = trans + (size_t)(sl + 1) * P.potNx * P.potNy;
            QS_TRY(launch_rows(ra, ROW_MID, s));
        }
    }
    if (exit_waves) QS_TRY(launch_rows(ra, ROW_LAST, s));
    if (wantDet) {
        const double scale = (double)P.electronScale / ((double)(nx * ny) * (double)(nx * ny));
        for (int t = 0; t < nT; t++) {
            if (lastWriter[t] < 0) continue;
            QS_TRY(launch_det_finalize(d_part + (size_t)t * partPerT, npos, ntiles, ndet, scale, d_pos + 2 * npos,
                                       d_pos + 3 * npos, P.scanYN, npix, det_images + (size_t)t * ndet * npix, s));
        }
    }
    return QS_OK;
}
