// qs_api.cu -- the C ABI (include/qstem_gpu.h): contexts, argument checks,
// host-side planning and the launch sequences of the multislice path.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "qs_fft.cuh"
#include "qs_internal.h"
#include "qs_zorder.h"

constexpr int kMaxBufs = 32;

struct qs_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    // reusable device buffers, grown on demand
    void* buf[kMaxBufs] = {};
    size_t cap[kMaxBufs] = {};
    // profiling
    bool profile = false;
    long long launch_base = 0;
    std::vector<cudaEvent_t> pool;       // event pool
    size_t pool_used = 0;
    std::vector<std::pair<size_t, size_t>> row_ev, col_ev;  // indices into pool
    double row_bytes = 0, col_bytes = 0;
    // projected-potential tables built so far, keyed by everything they depend on
    struct LutKey {
        int Z, charged;
        double B;
        float rx, ry, dz, R;
        bool operator<(const LutKey& o) const {
            return std::tie(Z, charged, B, rx, ry, dz, R) < std::tie(o.Z, o.charged, o.B, o.rx, o.ry, o.dz, o.R);
        }
    };
    std::map<LutKey, float*> luts;
    // QS_GRAPH: slice loops captured as CUDA graphs, keyed by every value
    // their launches bake in (a few, oldest dropped first)
    struct GraphEntry {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec = nullptr;
        int launches = 0;   // kernels in the graph
    };
    std::vector<GraphEntry> graphs;
    // pinned host staging of uploads: one buffer per kind, refilled once the
    // copy queued from it (the event recorded after it) has run, so that the
    // host can plan the next call while the device still works on this one
    struct Pinned {
        void* p = nullptr;
        size_t cap = 0;
        cudaEvent_t ev = nullptr;
        bool pending = false;
    };
    Pinned pin[5];
    // the scatter's knot thresholds in B_KNOTS were made for this (dr, Nr)
    double knots_dr = -1.0;
    int knots_Nr = 0;
    // knot thresholds computed so far (host), keyed by (dr, Nr): instances
    // of different samplings in turn reuse them
    std::map<std::pair<double, int>, std::vector<double>> knots_host;
};

namespace qs {

static thread_local std::string g_err;
void set_error(const std::string& m) { g_err = m; }
std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }

static int ev_record(qs_ctx* c, size_t* idx) {
    if (c->pool_used == c->pool.size()) {
        cudaEvent_t e;
        QS_CUDA_TRY(cudaEventCreate(&e));
        c->pool.push_back(e);
    }
    *idx = c->pool_used++;
    QS_CUDA_TRY(cudaEventRecord(c->pool[*idx], c->stream));
    return QS_OK;
}

enum Buf {
    B_WAVES, B_PROBE, B_PARTIAL, B_POS, B_TABLES, B_TILES, B_TRANS, B_OUT1, B_OUT2, B_OUT3, B_JOBS, B_LUTS,
    B_LUTPTR, B_SUM, B_DIFF_IN, B_ADJ, B_TEM, B_CBED, B_DFT, B_BAND, B_VREAL, B_KNOTS, B_STEPS, NBUF
};
static_assert(NBUF <= kMaxBufs, "context buffer table too small");
enum Pin { P_JOBS, P_LUTPTR, P_BAND, P_TABLES, P_KNOTS };

// Pinned host memory of `bytes` for staging kind `which`; waits only for the
// previous copy from the same buffer.
static int stage(qs_ctx* c, int which, size_t bytes, void** out) {
    qs_ctx::Pinned& b = c->pin[which];
    if (b.pending) {
        QS_CUDA_TRY(cudaEventSynchronize(b.ev));
        b.pending = false;
    }
    if (b.cap < bytes) {
        if (b.p) cudaFreeHost(b.p);
        b.p = nullptr;
        b.cap = 0;
        QS_CUDA_TRY(cudaMallocHost(&b.p, bytes));
        b.cap = bytes;
    }
    if (!b.ev) QS_CUDA_TRY(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming));
    *out = b.p;
    return QS_OK;
}

// Queue the copy of `bytes` from staging buffer `which` (filled by the caller
// after stage()) to device address dst.
static int stage_copy(qs_ctx* c, int which, void* dst, size_t bytes) {
    qs_ctx::Pinned& b = c->pin[which];
    QS_CUDA_TRY(cudaMemcpyAsync(dst, b.p, bytes, cudaMemcpyHostToDevice, c->stream));
    QS_CUDA_TRY(cudaEventRecord(b.ev, c->stream));
    b.pending = true;
    return QS_OK;
}

static int upload(qs_ctx* c, int which, void* dst, const void* src, size_t bytes) {
    void* h = nullptr;
    QS_TRY(stage(c, which, bytes, &h));
    std::memcpy(h, src, bytes);
    return stage_copy(c, which, dst, bytes);
}

static int ensure(qs_ctx* c, int which, size_t bytes, void** out) {
    if (bytes == 0) bytes = 16;
    if (c->cap[which] < bytes) {
        if (c->buf[which]) {
            cudaStreamSynchronize(c->stream);
            cudaFree(c->buf[which]);
            c->buf[which] = nullptr;
            c->cap[which] = 0;
        }
        cudaError_t e = cudaMalloc(&c->buf[which], bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("device allocation of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? QS_ERR_NOMEM : QS_ERR_CUDA;
        }
        c->cap[which] = bytes;
    }
    *out = c->buf[which];
    return QS_OK;
}

int check_params(const qs_params* p) {
    if (!p) { set_error("params is NULL"); return QS_ERR_ARG; }
    if (p->nx < 1 || p->ny < 1 || p->slices < 1 || p->potNx < p->nx || p->potNy < p->ny) {
        set_error("inconsistent grid sizes (nx, ny, potNx, potNy, slices)");
        return QS_ERR_ARG;
    }
    if (!(p->resolutionX > 0) || !(p->resolutionY > 0) || !(p->sliceThickness > 0) || !(p->v0 > 0)) {
        set_error("resolution, slice thickness and v0 must be positive");
        return QS_ERR_ARG;
    }
    if (p->cellDiv < 1) { set_error("cellDiv must be >= 1"); return QS_ERR_ARG; }
    if (p->mulsRepeat1 < 0 || p->mulsRepeat2 < 0) { set_error("mulsRepeat1/2 must be >= 0"); return QS_ERR_ARG; }
    if (p->outputInterval < 1) { set_error("outputInterval must be >= 1"); return QS_ERR_ARG; }
    if (p->detectorNum < 0 || p->detectorNum > QS_MAX_DETECTORS) { set_error("detectorNum out of range"); return QS_ERR_ARG; }
    return QS_OK;
}

int check_raster(const qs_params& p, const qs_batch& b, bool wantDetPixels) {
    const bool needRaster = !(b.iPosX && b.iPosY) || (wantDetPixels && !(b.detPosX && b.detPosY));
    if (needRaster && (p.scanXN < 1 || p.scanYN < 1)) {
        set_error("the batch takes positions or detector pixels from the scan raster, which needs "
                  "scanXN, scanYN >= 1");
        return QS_ERR_ARG;
    }
    return QS_OK;
}

double wavelength(double kev) { return 12.3984244 / std::sqrt(kev * (2 * 510.99906 + kev)); }

PropTables prop_tables(const qs_params& p) {
    PropTables t;
    const int nx = p.nx, ny = p.ny;
    const float ax = p.resolutionX * nx, by = p.resolutionY * ny;
    const float scale = (float)(p.sliceThickness * 3.14159265358979);
    const float wavlen = (float)wavelength(p.v0);
    t.kx2.resize(nx); t.px.resize(nx); t.ky2.resize(ny); t.py.resize(ny);
    for (int i = 0; i < nx; i++) {
        float k = (i > nx / 2) ? (float)(i - nx) / ax : (float)i / ax;
        t.kx2[i] = k * k;
        float a = scale * (t.kx2[i] * wavlen);
        t.px[i] = make_float2(cosf(a), -sinf(a));
    }
    for (int i = 0; i < ny; i++) {
        float k = (i > ny / 2) ? (float)(i - ny) / by : (float)i / by;
        t.ky2[i] = k * k;
        float a = scale * (t.ky2[i] * wavlen);
        t.py[i] = make_float2(cosf(a), -sinf(a));
    }
    float k2max = nx / (2.0f * ax);
    if (ny / (2.0f * by) < k2max) k2max = ny / (2.0f * by);
    k2max = (float)(2.0 / 3.0 * k2max);
    t.k2max = k2max * k2max;
    return t;
}

Band band_tiles(const PropTables& t, int ny, int colTile) {
    Band b;
    b.yA = -1;
    b.yB = ny;
    for (int iy = 0; iy <= ny / 2; iy++) if (t.ky2[iy] < t.k2max) b.yA = iy;
    for (int iy = ny - 1; iy > ny / 2; iy--) if (t.ky2[iy] < t.k2max) b.yB = iy;
    for (int iy = 0; iy < ny; iy++)
        if ((t.ky2[iy] < t.k2max) != (iy <= b.yA || iy >= b.yB)) { b.yA = ny; b.yB = ny; break; }
    for (int c0 = 0; c0 < ny; c0 += colTile) {
        bool any = false;
        for (int k = c0; k < c0 + colTile && k < ny; k++) any |= (k <= b.yA || k >= b.yB);
        if (any) b.tiles.push_back(c0);
    }
    return b;
}

static int thickness_count(const qs_params& p) { return (p.slices * p.cellDiv) / p.outputInterval + 1; }

// The control flow of make3DSlices' atom loop (stem3/stemlib.cpp:678-1213)
// reduced to one job per contributing atom: atoms sorted by z (stable), the
// vacancy skip, the non-periodic z cut-offs, the pixel box and the slice
// range.  lutKeys lists (Z*2 + charged, B) in first-use order; B is the
// Debye-Waller factor of the element's first contributing atom, as the
// reference's per-element LUT cache keeps it (:1417).
static void plan_atoms(const qs_params& P, const qs_atom* atoms, int natom, std::vector<AtomJob>& jobs,
                       std::vector<std::pair<int, double>>& lutKeys, int slab = 0) {
    std::vector<int> order;
    z_order(natom, [&](int i) { return atoms[i].z; }, order);
    std::vector<qs_atom> at(natom);
    for (int i = 0; i < natom; i++) at[i] = atoms[order[i]];
    const float cz = P.sliceThickness * (float)P.slices;
    const float dx = P.resolutionX, dy = P.resolutionY, dzs = P.sliceThickness;
    const int iRadX = (int)ceilf(P.atomRadius / dx), iRadY = (int)ceilf(P.atomRadius / dy);
    const int iRadZ = (int)ceilf(P.atomRadius / dzs);
    jobs.clear();
    lutKeys.clear();
    std::map<int, int> lutIndex;          // key Z*2+charged -> index
    auto atomz = [&](int i) {
        // slab `slab` sees the atoms shifted down by slab * cz (stem3/stemlib.cpp:709-713)
        float z = (float)((double)(at[i].z - cz * (float)slab + P.czOffset) -
                          0.5 * P.sliceThickness * (1 - P.centerSlices));
        z -= P.sliceThickness;
        return z;
    };
    for (int ia = 0; ia < natom; ia++) {
        while (ia < natom && at[ia].Znum == 0) ia++;
        if (ia >= natom) break;
        float atomZ = atomz(ia);
        if (P.nonPeriodZ) {
            if (atomZ - P.atomRadius > cz) break;
            do {
                if (atomZ + P.atomRadius + P.sliceThickness >= 0) break;
                ++ia;
                atomZ = atomz(ia);
            } while (ia < natom - 1);
        }
        const float atomX = at[ia].x - P.potOffsetX, atomY = at[ia].y - P.potOffsetY;
        const int iAtomX = (int)floorf(atomX / dx), iAtomY = (int)floorf(atomY / dy);
        atomZ += P.sliceThickness;
        const int iAtomZ = (int)floor(atomZ / dzs + 0.5);
        AtomJob J;
        if (P.nonPeriod) {
            J.iax0 = std::max(iAtomX - iRadX, 0);
            J.iax1 = std::min(iAtomX + iRadX, P.potNx - 1);
            J.iay0 = std::max(iAtomY - iRadY, 0);
            J.iay1 = std::min(iAtomY + iRadY, P.potNy - 1);
            if (!((J.iax0 < P.potNx) && (J.iax1 >= 0) && (J.iay0 < P.potNy) && (J.iay1 >= 0))) continue;
        } else {
            J.iax0 = iAtomX - iRadX;
            J.iax1 = iAtomX + iRadX - 1;
            J.iay0 = iAtomY - iRadY;
            J.iay1 = iAtomY + iRadY - 1;
        }
        J.iaz0 = iAtomZ - iRadZ < 0 ? -iAtomZ : -iRadZ;
        J.iaz1 = iAtomZ + iRadZ >= P.slices ? P.slices - iAtomZ - 1 : iRadZ;
        if (!((iAtomZ + J.iaz0 < P.slices) && (iAtomZ + J.iaz1 >= 0))) continue;
        const int Z = at[ia].Znum;
        if (Z < 1 || Z >= 93) continue;
        if (J.iax1 < J.iax0 || J.iay1 < J.iay0 || J.iaz1 < J.iaz0) continue;
        const double B = P.tds ? 0.0 : at[ia].dw;
        for (int charged = 0; charged < 2; charged++) {
            if (charged && at[ia].q == 0) break;
            const int key = Z * 2 + charged;
            if (!lutIndex.count(key)) {
                lutIndex[key] = (int)lutKeys.size();
                lutKeys.push_back({key, B});
            }
        }
        J.index = order[ia];
        J.atomX = atomX;
        J.atomY = atomY;
        J.atomZ = atomZ;
        J.q = at[ia].q;
        J.iAtomZ = iAtomZ;
        J.lut = lutIndex[Z * 2];
        J.lutq = at[ia].q != 0 ? lutIndex[Z * 2 + 1] : -1;
        jobs.push_back(J);
    }

}

// The atoms of make3DSlices' periodic 2-D branch (stem3/stemlib.cpp:709-731
// for the atom z, :1215-1262): z-sorted, vacancies skipped, the 2-D z offset
// (+ dz/2 where the 3-D branch takes - dz), one slice floor(atomZ/dz) per
// atom (atoms whose slice lies outside the stack are left out: the
// reference writes outside its array there), the box, table offsets and
// bilinear weights formed as the reference forms them.  keys: (Z, B) of
// every element's table, B that of its first atom in z order.
static void plan_atoms_2d(const qs_params& P, const qs_atom* atoms, int natom, std::vector<Atom2DJob>& jobs,
                          std::vector<std::pair<int, double>>& keys, int slab = 0) {
    std::vector<int> order;
    z_order(natom, [&](int i) { return atoms[i].z; }, order);
    const float cz = P.sliceThickness * (float)P.slices;
    const float dx = P.resolutionX, dy = P.resolutionY, dzs = P.sliceThickness;
    const int iRadX = (int)ceilf(P.atomRadius / dx), iRadY = (int)ceilf(P.atomRadius / dy);
    jobs.clear();
    keys.clear();
    std::map<int, int> index;
    auto atomz = [&](int i) {
        float z = (float)((double)(atoms[order[i]].z - cz * (float)slab + P.czOffset) -
                          0.5 * P.sliceThickness * (1 - P.centerSlices));
        return (float)((double)z + 0.5 * P.sliceThickness);
    };
    for (int ia = 0; ia < natom; ia++) {
        while (ia < natom && atoms[order[ia]].Znum == 0) ia++;
        if (ia >= natom) break;
        float atomZ = atomz(ia);
        if (P.nonPeriodZ) {
            if (atomZ > cz) break;
            do {
                if (atomZ >= 0) break;
                ++ia;
                atomZ = atomz(ia);
            } while (ia < natom - 1);
        }
        const qs_atom& A = atoms[order[ia]];
        const float atomX = A.x - P.potOffsetX, atomY = A.y - P.potOffsetY;
        const int iAtomX = (int)floorf(atomX / dx), iAtomY = (int)floorf(atomY / dy);
        const int iAtomZ = (int)floor(atomZ / dzs);
        const int Z = A.Znum;
        if (Z < 1 || Z >= 93 || iAtomZ < 0 || iAtomZ >= P.slices) continue;
        if (!index.count(Z)) {
            index[Z] = (int)keys.size();
            keys.push_back({Z, P.tds ? 0.0 : A.dw});
        }
        Atom2DJob J;
        J.lut = index[Z];
        J.iAtomZ = iAtomZ;
        J.iax0 = iAtomX - iRadX;
        J.iay0 = iAtomY - iRadY;
        // (-iax0' + (atomX/dx - (iRadX - 2 potNx))) * OVERSAMP with the
        // reference's iax0' = iax0 + 2 potNx, the quotient in float
        double ddx = (-(double)(J.iax0 + 2 * P.potNx) + (atomX / dx - (double)(iRadX - 2 * P.potNx))) * 2.0;
        double ddy = (-(double)(J.iay0 + 2 * P.potNy) + (atomY / dy - (double)(iRadY - 2 * P.potNy))) * 2.0;
        J.iOffsX = (int)floor(ddx);
        J.iOffsY = (int)floor(ddy);
        ddx -= (double)J.iOffsX;
        ddy -= (double)J.iOffsY;
        J.s22 = (1 - ddx) * (1 - ddy);
        J.s21 = (1 - ddx) * ddy;
        J.s12 = ddx * (1 - ddy);
        J.s11 = ddx * ddy;
        jobs.push_back(J);
    }
}

// Device LUT pointers for lutKeys, built on first use and kept by the context.
static int prepare_luts(qs_ctx* c, const qs_params& P, const std::vector<std::pair<int, double>>& lutKeys,
                        const float* const** d_ptrs, int* Nz, int* Nr, int* nzSub) {
    QS_TRY(build_lut(P, 1, 0.0, 0, nullptr, Nz, Nr, nzSub, c->stream));
    const size_t lutElems = (size_t)(*Nz) * (*Nr);
    void* dp = nullptr;
    QS_TRY(ensure(c, B_LUTPTR, sizeof(float*) * std::max<size_t>(lutKeys.size(), 1), &dp));
    std::vector<const float*> ptrs(lutKeys.size());
    for (size_t k = 0; k < lutKeys.size(); k++) {
        // tables depend only on the element, charge flag, B and the sampling;
        // the context keeps them across calls (frozen-phonon runs reuse them)
        const qs_ctx::LutKey key{lutKeys[k].first / 2, lutKeys[k].first % 2, lutKeys[k].second,
                                 P.resolutionX, P.resolutionY, P.sliceThickness, P.atomRadius};
        auto it = c->luts.find(key);
        if (it == c->luts.end()) {
            float* d = nullptr;
            cudaError_t e = cudaMalloc(&d, sizeof(float) * lutElems);
            if (e != cudaSuccess) {
                cudaGetLastError();
                set_error(std::string("LUT allocation failed: ") + cudaGetErrorString(e));
                return QS_ERR_NOMEM;
            }
            const int rc = build_lut(P, key.Z, key.B, key.charged, d, nullptr, nullptr, nullptr, c->stream);
            if (rc != QS_OK) {
                cudaStreamSynchronize(c->stream);
                cudaFree(d);
                return rc;
            }
            it = c->luts.emplace(key, d).first;
            // build_lut's host tables (once per element and sampling) must
            // outlive its copies
            QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
        }
        ptrs[k] = it->second;
    }
    if (!ptrs.empty()) QS_TRY(upload(c, P_LUTPTR, dp, ptrs.data(), sizeof(float*) * ptrs.size()));
    *d_ptrs = (const float* const*)dp;
    return QS_OK;
}

// Bytes of values, appended to a graph key.
struct KeyBytes {
    std::vector<unsigned char> b;
    template <class T>
    KeyBytes& add(const T& v) {
        const unsigned char* q = reinterpret_cast<const unsigned char*>(&v);
        b.insert(b.end(), q, q + sizeof(T));
        return *this;
    }
};

}  // namespace qs

using namespace qs;

// ====================================================================== C ABI
extern "C" {

const char* qs_last_error(void) { return g_err.c_str(); }
int qs_abi_version(void) { return QS_ABI_VERSION; }

int qs_ctx_create(int device, qs_ctx** out) {
    if (!out) { set_error("out is NULL"); return QS_ERR_ARG; }
    *out = nullptr;
    int n = 0;
    QS_CUDA_TRY(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) { set_error("no such CUDA device"); return QS_ERR_ARG; }
    QS_CUDA_TRY(cudaSetDevice(device));
    qs_ctx* c = new qs_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        return QS_ERR_CUDA;
    }
    *out = c;
    return QS_OK;
}

int qs_ctx_destroy(qs_ctx* c) {
    if (!c) return QS_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    for (auto& g : c->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto& kv : c->luts) cudaFree(kv.second);
    for (auto& b : c->pin) {
        if (b.p) cudaFreeHost(b.p);
        if (b.ev) cudaEventDestroy(b.ev);
    }
    for (int i = 0; i < kMaxBufs; i++)
        if (c->buf[i]) cudaFree(c->buf[i]);
    cudaStreamDestroy(c->stream);
    delete c;
    return QS_OK;
}

void* qs_ctx_stream(qs_ctx* c) { return c ? (void*)c->stream : nullptr; }

int qs_ctx_profile(qs_ctx* c, int enable) {
    if (!c) { set_error("ctx is NULL"); return QS_ERR_ARG; }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->profile = enable != 0;
    c->launch_base = g_launches.load();
    c->pool_used = 0;
    c->row_ev.clear();
    c->col_ev.clear();
    c->row_bytes = c->col_bytes = 0;
    return QS_OK;
}

int qs_ctx_stats(qs_ctx* c, qs_stats* out) {
    if (!c || !out) { set_error("null argument"); return QS_ERR_ARG; }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    std::memset(out, 0, sizeof(*out));
    out->launches = g_launches.load() - c->launch_base;
    out->row_launches = (long long)c->row_ev.size();
    out->col_launches = (long long)c->col_ev.size();
    for (auto& pr : c->row_ev) {
        float ms = 0;
        QS_CUDA_TRY(cudaEventElapsedTime(&ms, c->pool[pr.first], c->pool[pr.second]));
        out->row_ms += ms;
    }
    for (auto& pr : c->col_ev) {
        float ms = 0;
        QS_CUDA_TRY(cudaEventElapsedTime(&ms, c->pool[pr.first], c->pool[pr.second]));
        out->col_ms += ms;
    }
    out->row_bytes = c->row_bytes;
    out->col_bytes = c->col_bytes;
    return QS_OK;
}

int qs_params_finalize(qs_params* p) {
    if (!p) { set_error("params is NULL"); return QS_ERR_ARG; }
    const double wl = wavelength(p->v0);
    for (int i = 0; i < p->detectorNum && i < QS_MAX_DETECTORS; i++) {
        qs_detector* d = &p->detectors[i];
        d->k2Inside = (float)(std::sin(d->rInside * 0.001) / wl);
        d->k2Outside = (float)(std::sin(d->rOutside * 0.001) / wl);
        d->k2Inside *= d->k2Inside;
        d->k2Outside *= d->k2Outside;
    }
    return QS_OK;
}

int qs_thickness_count(const qs_params* p) {
    if (!p || p->outputInterval < 1) return 0;
    return thickness_count(*p);
}

int qs_lut_build(qs_ctx* c, const qs_params* p, int Z, double B, int charged, float* out, int* Nz, int* Nr,
                 int* nzSub, unsigned flags) {
    if (!c) { set_error("ctx is NULL"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    QS_CUDA_TRY(cudaSetDevice(c->device));
    int nz = 0, nr = 0, ns = 0;
    QS_TRY(build_lut(*p, Z, B, charged, nullptr, &nz, &nr, &ns, c->stream));
    if (Nz) *Nz = nz;
    if (Nr) *Nr = nr;
    if (nzSub) *nzSub = ns;
    if (!out) return QS_OK;
    float* dst = out;
    if (flags & QS_HOST_IO) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT1, sizeof(float) * (size_t)nz * nr, &d));
        dst = (float*)d;
    }
    QS_TRY(build_lut(*p, Z, B, charged, dst, nullptr, nullptr, nullptr, c->stream));
    if (flags & QS_HOST_IO) {
        QS_CUDA_TRY(cudaMemcpyAsync(out, dst, sizeof(float) * (size_t)nz * nr, cudaMemcpyDeviceToHost, c->stream));
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else if (flags & QS_SYNC) {
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    return QS_OK;
}

int qs_slices_build(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, float* trans_out,
                    unsigned flags) {
    return qs_slab_build(c, p, atoms, natom, 0, trans_out, flags);
}

}  // extern "C"

namespace {
// a custom scattering-factor table (readSFactLUT, stem3/stem3.cpp:555-600)
struct CustomSF {
    const double* k;
    int nk;
    const int* Z;
    const double* f;
    int nkinds;
};
}  // namespace

// qs_slab_build, and with a custom table make3DSlicesFT in place of
// make3DSlices
static int slab_build(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, int slab, float* trans_out,
                      unsigned flags, const CustomSF* cs) {
    if (!c || !trans_out || (natom > 0 && !atoms)) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    if (slab < 0 || slab >= p->cellDiv) {
        set_error("slab " + std::to_string(slab) + " outside 0.." + std::to_string(p->cellDiv - 1));
        return QS_ERR_ARG;
    }
    if (!cs && !p->fftpotential) {
        set_error("only the FFT-integrated potential (one time integration) is supported");
        return QS_ERR_UNSUPPORTED;
    }
    if (!cs && !p->potential3D) {
        // the 2-D potential: its periodic branch only (the non-periodic one
        // reads its table outside the array for atoms near the edges), and
        // tables at least as wide in x as in y (the reference bounds x by the
        // y width and reads past a narrower table)
        const int nx2 = 2 * 2 * (int)ceilf(p->atomRadius / p->resolutionX);
        const int ny2 = 2 * 2 * (int)ceilf(p->atomRadius / p->resolutionY);
        if (p->nonPeriod || nx2 < ny2) {
            set_error(p->nonPeriod ? "the 2-D potential needs a periodic potential array (periodicXY)"
                                   : "the 2-D potential needs ceil(atomRadius/dx) >= ceil(atomRadius/dy)");
            return QS_ERR_UNSUPPORTED;
        }
    }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    const qs_params& P = *p;
    const size_t nTrans = (size_t)P.slices * P.potNx * P.potNy;
    float2* trans = (float2*)trans_out;
    if (flags & QS_HOST_IO) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_TRANS, sizeof(float2) * nTrans, &d));
        trans = (float2*)d;
    }
    // make3DSlices' sums go to a real array first (the phase grating, or
    // for QS_OUT_POTENTIAL a plain copy, fills the complex stack from it)
    void* dvr = nullptr;
    QS_TRY(ensure(c, B_VREAL, sizeof(float) * nTrans, &dvr));
    float* Vr = (float*)dvr;
    QS_CUDA_TRY(cudaMemsetAsync(Vr, 0, sizeof(float) * nTrans, c->stream));

    std::vector<AtomJob> jobs;
    std::vector<std::pair<int, double>> lutKeys;
    if (cs) {
        // make3DSlicesFT: every slab's stack is slab 0's (the reference's
        // slab counter is a local of the function, restarted at 0)
        QS_TRY(build_custom_potential(P, atoms, natom, cs->k, cs->nk, cs->Z, cs->f, cs->nkinds, Vr, c->stream));
    } else if (!P.potential3D) {
        // make3DSlices' periodic 2-D branch
        std::vector<Atom2DJob> jobs2;
        plan_atoms_2d(P, atoms, natom, jobs2, lutKeys, slab);
        if (!jobs2.empty()) {
            int nx2 = 0, ny2 = 0;
            QS_TRY(build_lut2d(P, 1, 0.0, nullptr, &nx2, &ny2, c->stream));
            void* dp = nullptr;
            QS_TRY(ensure(c, B_LUTPTR, sizeof(float*) * lutKeys.size(), &dp));
            std::vector<const float*> ptrs(lutKeys.size());
            for (size_t k = 0; k < lutKeys.size(); k++) {
                // cached with the 3-D tables (charge flag 2 marks a 2-D table)
                const qs_ctx::LutKey key{lutKeys[k].first, 2, lutKeys[k].second, P.resolutionX, P.resolutionY,
                                         0.f, P.atomRadius};
                auto it = c->luts.find(key);
                if (it == c->luts.end()) {
                    float* d = nullptr;
                    cudaError_t e = cudaMalloc(&d, sizeof(float) * (size_t)nx2 * ny2);
                    if (e != cudaSuccess) {
                        cudaGetLastError();
                        set_error(std::string("2-D table allocation failed: ") + cudaGetErrorString(e));
                        return QS_ERR_NOMEM;
                    }
                    const int rc = build_lut2d(P, key.Z, key.B, d, nullptr, nullptr, c->stream);
                    if (rc != QS_OK) {
                        cudaStreamSynchronize(c->stream);
                        cudaFree(d);
                        return rc;
                    }
                    it = c->luts.emplace(key, d).first;
                    // the builder's host tables must outlive their copies
                    QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
                }
                ptrs[k] = it->second;
            }
            QS_TRY(upload(c, P_LUTPTR, dp, ptrs.data(), sizeof(float*) * ptrs.size()));
            void* dj = nullptr;
            QS_TRY(ensure(c, B_JOBS, sizeof(Atom2DJob) * jobs2.size(), &dj));
            QS_TRY(upload(c, P_JOBS, dj, jobs2.data(), sizeof(Atom2DJob) * jobs2.size()));
            const int iRadX = (int)ceilf(P.atomRadius / P.resolutionX), iRadY = (int)ceilf(P.atomRadius / P.resolutionY);
            QS_TRY(launch_scatter2d((const Atom2DJob*)dj, (int)jobs2.size(), (const float* const*)dp, ny2, 2 * iRadX,
                                    2 * iRadY, P, Vr, c->stream));
        }
    } else {
        plan_atoms(P, atoms, natom, jobs, lutKeys, slab);
    }

    if (!jobs.empty()) {
        int Nz = 0, Nr = 0, ns = 0;
        const float* const* d_luts = nullptr;
        QS_TRY(prepare_luts(c, P, lutKeys, &d_luts, &Nz, &Nr, &ns));
        void* dj = nullptr;
        QS_TRY(ensure(c, B_JOBS, sizeof(AtomJob) * jobs.size(), &dj));
        QS_TRY(upload(c, P_JOBS, dj, jobs.data(), sizeof(AtomJob) * jobs.size()));
        void* dk = nullptr;
        QS_TRY(ensure(c, B_KNOTS, sizeof(double) * (Nr + 1), &dk));
        const double dr = (double)(P.resolutionX / 2);  // make3DSlices' dr (stem3/stemlib.cpp:576)
        if (c->knots_dr != dr || c->knots_Nr != Nr) {
            std::vector<double>& knots = c->knots_host[{dr, Nr}];
            if (knots.empty()) scatter_knots(dr, Nr, knots);
            QS_TRY(upload(c, P_KNOTS, dk, knots.data(), sizeof(double) * knots.size()));
            c->knots_dr = dr;
            c->knots_Nr = Nr;
        }
        bool charged = false;
        for (const AtomJob& J : jobs) charged |= J.lutq >= 0;
        QS_TRY(launch_scatter((const AtomJob*)dj, (int)jobs.size(), charged, d_luts, Nz, Nr, ns, P,
                              (const double*)dk, Vr, c->stream));
    }

    if (flags & QS_OUT_POTENTIAL) {
        QS_TRY(launch_expand_real(Vr, trans, nTrans, c->stream));
    } else {
        // initSTEMSlices (stem3/stemlib.cpp:2280-2336)
        const double mm0 = (double)(1.0f + P.v0 / 511.0f);
        QS_TRY(launch_grating_from_real(Vr, trans, nTrans, mm0 * wavelength(P.v0), c->stream));
        // line FFTs where they exist, DFT matrix products otherwise
        const bool lines = line_supported(P.potNx) && line_supported(P.potNy);
        if (P.bandlimittrans) {
            const int nx = P.potNx, ny = P.potNy;
            float2* scr = nullptr;
            int scrSlices = 0;
            if (!lines) {
                scrSlices = std::min(P.slices, 16);
                void* d = nullptr;
                QS_TRY(ensure(c, B_DFT, sizeof(float2) * (size_t)nx * ny * scrSlices, &d));
                scr = (float2*)d;
            }
            auto xform = [&](bool inverse) -> int {
                return lines ? fft2d(trans, nx, ny, P.slices, inverse, c->stream)
                             : dft2d(trans, nx, ny, P.slices, inverse, scr, scrSlices, c->stream);
            };
            std::vector<float> kx2(nx), ky2(ny);
            for (int ix = 0; ix < nx; ix++) {
                float kx = (ix > nx / 2) ? (float)(ix - nx) / P.potSizeX : (float)ix / P.potSizeX;
                kx2[ix] = kx * kx;
            }
            for (int iy = 0; iy < ny; iy++) {
                float ky = (iy > ny / 2) ? (float)(iy - ny) / P.by : (float)iy / P.potSizeY;
                ky2[iy] = ky * ky;
            }
            float k2max = nx / (2.0f * P.potSizeX), tt = ny / (2.0f * P.potSizeY);
            if (tt < k2max) k2max = tt;
            k2max = (float)((2.0f / 3.0f) * k2max);
            k2max = k2max * k2max;
            void* dt = nullptr;
            if (lines) {
                // FFT_y storing the in-band columns, one column pass over
                // their tiles (FFT_x, mask and 1/N, IFFT_x), IFFT_y
                const int Cw = col_tile_width(nx);
                PropTables bt;
                bt.ky2 = ky2;
                bt.k2max = k2max;
                const Band band = band_tiles(bt, ny, Cw);
                const int ntl = (int)band.tiles.size();
                const size_t bytes = sizeof(float) * (nx + ny) + sizeof(float2) * (nx + ny) + sizeof(int) * ntl;
                QS_TRY(ensure(c, B_BAND, bytes, &dt));
                void* hbuf = nullptr;
                QS_TRY(stage(c, P_BAND, bytes, &hbuf));
                float* hk = (float*)hbuf;
                std::copy(kx2.begin(), kx2.end(), hk);
                std::copy(ky2.begin(), ky2.end(), hk + nx);
                float2* hp = (float2*)(hk + nx + ny);
                const float sc = (float)(1.0 / (nx * ny));
                for (int i = 0; i < nx; i++) hp[i] = make_float2(sc, 0.f);
                for (int i = 0; i < ny; i++) hp[nx + i] = make_float2(1.f, 0.f);
                int* ht = (int*)(hp + nx + ny);
                for (int k = 0; k < ntl; k++) ht[k] = band.tiles[k];
                QS_TRY(stage_copy(c, P_BAND, dt, bytes));
                const float* dk = (const float*)dt;
                const float2* dp = (const float2*)(dk + nx + ny);
                QS_TRY(bandlimit_lines(trans, nx, ny, P.slices, dk, dk + nx, dp, dp + nx, (const int*)(dp + nx + ny),
                                       ntl, band.yA, band.yB, k2max, c->stream));
            } else {
                QS_TRY(ensure(c, B_TABLES, sizeof(float) * (nx + ny), &dt));
                std::vector<float> both(kx2);
                both.insert(both.end(), ky2.begin(), ky2.end());
                QS_TRY(upload(c, P_TABLES, dt, both.data(), sizeof(float) * both.size()));
                QS_TRY(xform(false));
                QS_TRY(launch_bandlimit_mask(trans, P.slices, nx, ny, (float*)dt, (float*)dt + nx, k2max,
                                             1.0 / (nx * ny), c->stream));
                QS_TRY(xform(true));
            }
        }
    }
    if (flags & QS_HOST_IO) {
        QS_CUDA_TRY(cudaMemcpyAsync(trans_out, trans, sizeof(float2) * nTrans, cudaMemcpyDeviceToHost, c->stream));
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else if (flags & QS_SYNC) {
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    return QS_OK;
}

extern "C" {

int qs_slab_build(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, int slab, float* trans_out,
                  unsigned flags) {
    return slab_build(c, p, atoms, natom, slab, trans_out, flags, nullptr);
}

int qs_slices_build_custom(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, const double* k, int nk,
                           const int* Z, const double* f, int nkinds, float* trans_out, unsigned flags) {
    if (!k || !Z || !f || nk < 4 || nkinds < 1) {
        set_error("custom scattering factors: k, Z and f tables needed (nk >= 4, nkinds >= 1)");
        return QS_ERR_ARG;
    }
    const CustomSF cs{k, nk, Z, f, nkinds};
    return slab_build(c, p, atoms, natom, 0, trans_out, flags, &cs);
}

static int probe_into(qs_ctx* c, const qs_params& P, double dx, double dy, float2* w) {
    if (!line_supported(P.nx) || !line_supported(P.ny)) {
        set_error("probe: nx, ny must be in {64,128,256,384,512,768,1024}");
        return QS_ERR_UNSUPPORTED;
    }
    void* ds = nullptr;
    QS_TRY(ensure(c, B_SUM, sizeof(double) * 2, &ds));
    QS_TRY(launch_probe_kspace(P, dx, dy, w, c->stream));
    QS_TRY(fft2d(w, P.nx, P.ny, 1, true, c->stream));
    QS_TRY(launch_probe_realspace(P, dx, dy, w, (double*)ds, c->stream));
    QS_TRY(launch_scale_by_sum(w, (size_t)P.nx * P.ny, (double*)ds, (double)P.nx * (double)P.ny, c->stream));
    return QS_OK;
}

int qs_probe(qs_ctx* c, const qs_params* p, double dx, double dy, float* wave, unsigned flags) {
    if (!c || !wave) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    QS_CUDA_TRY(cudaSetDevice(c->device));
    const size_t n = (size_t)p->nx * p->ny;
    float2* w = (float2*)wave;
    if (flags & QS_HOST_IO) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_PROBE, sizeof(float2) * n, &d));
        w = (float2*)d;
    }
    QS_TRY(probe_into(c, *p, dx, dy, w));
    if (flags & QS_HOST_IO) {
        QS_CUDA_TRY(cudaMemcpyAsync(wave, w, sizeof(float2) * n, cudaMemcpyDeviceToHost, c->stream));
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    } else if (flags & QS_SYNC) {
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    }
    return QS_OK;
}

// The scan of qs_multislice_run, generalised to one transmission stack and
// one incident wave per wave of the batch (device arrays, consecutive waves
// transStride / probeStride elements apart; 0 = shared by all waves), which
// the TEM and CBED batch drivers use.

// Issue `work` (kernel launches and memsets on stream s) directly, or with
// QS_GRAPH through the context's graph cache: the first call with a key runs
// eagerly (first-use set-up happens outside any capture), the second is
// captured into a graph and launched, later ones replay the graph.
static int run_graphed(qs_ctx* c, cudaStream_t s, bool graph, const std::vector<unsigned char>& key,
                       const std::function<int()>& work) {
    if (!graph) return work();
    for (auto& g : c->graphs)
        if (g.key == key) {
            if (g.exec) {
                QS_CUDA_TRY(cudaGraphLaunch(g.exec, s));
                count_launch(g.launches);
                return QS_OK;
            }
            const long long before = g_launches.load();
            QS_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const int rc = work();
            cudaGraph_t gr = nullptr;
            const cudaError_t e = cudaStreamEndCapture(s, &gr);
            if (rc != QS_OK || e != cudaSuccess) {
                if (gr) cudaGraphDestroy(gr);
                cudaGetLastError();
                if (rc == QS_OK) set_error(std::string("graph capture failed: ") + cudaGetErrorString(e));
                return rc != QS_OK ? rc : QS_ERR_CUDA;
            }
            const cudaError_t ei = cudaGraphInstantiate(&g.exec, gr, 0);
            cudaGraphDestroy(gr);
            if (ei != cudaSuccess) {
                cudaGetLastError();
                g.exec = nullptr;
                set_error(std::string("graph instantiation failed: ") + cudaGetErrorString(ei));
                return QS_ERR_CUDA;
            }
            g.launches = (int)(g_launches.load() - before);
            g_launches -= g.launches;  // captured, not yet launched
            QS_CUDA_TRY(cudaGraphLaunch(g.exec, s));
            count_launch(g.launches);
            return QS_OK;
        }
    if (c->graphs.size() >= 8) {
        if (c->graphs.front().exec) {
            cudaStreamSynchronize(s);
            cudaGraphExecDestroy(c->graphs.front().exec);
        }
        c->graphs.erase(c->graphs.begin());
    }
    c->graphs.push_back({key, nullptr, 0});
    return work();
}

static int multislice_run_ex(qs_ctx* c, const qs_params* p, const float* trans_in, size_t transStride,
                             const float* probe_in, size_t probeStride, const qs_batch* batch, float* det_images,
                             float* diffpats, float* exit_waves, unsigned flags) {
    if (!c || !trans_in || !batch) { set_error("null argument"); return QS_ERR_ARG; }
    if ((transStride || probeStride) && ((flags & QS_HOST_IO) || (probeStride && !probe_in))) {
        set_error("per-wave stacks and incident waves must be device arrays");
        return QS_ERR_ARG;
    }
    QS_TRY(check_params(p));
    const qs_params& P = *p;
    if (!line_supported(P.nx) || !line_supported(P.ny)) {
        set_error("multislice: nx, ny must be in {64,128,256,384,512,768,1024}");
        return QS_ERR_UNSUPPORTED;
    }
    for (int d = 0; d < P.detectorNum; d++)
        if (P.detectors[d].shiftX != 0 || P.detectors[d].shiftY != 0) {
            set_error("multislice: shifted detectors are supported by qs_collect only");
            return QS_ERR_UNSUPPORTED;
        }
    const int npos = batch->npos;
    if (npos < 1) { set_error("batch has no positions"); return QS_ERR_ARG; }
    QS_TRY(check_raster(P, *batch, P.detectorNum > 0 && det_images != nullptr));
    QS_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int nx = P.nx, ny = P.ny, S = P.slices;
    const size_t N = (size_t)nx * ny;
    const bool host = (flags & QS_HOST_IO) != 0;
    const int nT = thickness_count(P);
    const int ndet = P.detectorNum;
    const int npix = P.scanXN * P.scanYN;

    // positions (host side)
    std::vector<int> px(npos), py(npos), dxp(npos), dyp(npos);
    for (int i = 0; i < npos; i++) {
        if (batch->iPosX && batch->iPosY) {
            px[i] = batch->iPosX[i];
            py[i] = batch->iPosY[i];
        } else {
            const int ix = i / P.scanYN, iy = i % P.scanYN;
            int x = (int)((float)ix * (P.scanXStop - P.scanXStart) / ((float)P.scanXN * P.resolutionX));
            int y = (int)((float)iy * (P.scanYStop - P.scanYStart) / ((float)P.scanYN * P.resolutionY));
            px[i] = std::min(x, P.potNx - nx);
            py[i] = std::min(y, P.potNy - ny);
        }
        // raster pixels (check_raster: scanYN >= 1 whenever they are used)
        dxp[i] = batch->detPosX ? batch->detPosX[i] : (P.scanYN > 0 ? i / P.scanYN : 0);
        dyp[i] = batch->detPosY ? batch->detPosY[i] : (P.scanYN > 0 ? i % P.scanYN : 0);
        if (px[i] < 0 || py[i] < 0 || px[i] > P.potNx - nx || py[i] > P.potNy - ny) {
            set_error("position " + std::to_string(i) + " puts the window outside the potential array");
            return QS_ERR_ARG;
        }
        if (ndet > 0 && det_images && (dxp[i] < 0 || dxp[i] >= P.scanXN || dyp[i] < 0 || dyp[i] >= P.scanYN)) {
            set_error("detector pixel of position " + std::to_string(i) + " outside the scan raster");
            return QS_ERR_ARG;
        }
    }

    // propagator tables, band, column tiles
    PropTables tb = prop_tables(P);
    const Band band = band_tiles(tb, ny, col_tile_width(nx));
    const int yA = band.yA, yB = band.yB;
    const std::vector<int>& tiles = band.tiles;
    const int ntiles = (int)tiles.size();

    // the steps of the wave: mulsRepeat2 passes through the cellDiv slabs
    // (doSTEM's slab loop, stem3/stem3.cpp:2795-2949), each slab's S
    // slices mulsRepeat1 times (runMulsSTEM's repeat loop,
    // stem3/stemlib.cpp:2403-2405); step a transmits stack slice
    // stepSlice[a] and hands collectIntensity the index
    // totalSliceCount + islice*(1 + repeat) (:2429)
    const int D = P.cellDiv, SA = S * D;
    const bool slabStacks = D > 1 && (flags & QS_SLAB_STACKS);
    std::vector<int> stepSlice, stepIndex;
    const int R1 = std::max(1, P.mulsRepeat1), R2 = std::max(1, P.mulsRepeat2);
    for (int pc = 0; pc < R2 * D; pc++)
        for (int r = 0; r < R1; r++)
            for (int i = 0; i < S; i++) {
                stepSlice.push_back((slabStacks ? (pc % D) * S : 0) + i);
                stepIndex.push_back(pc * S + i * (1 + r));
            }
    const int NS = (int)stepSlice.size();
    // output steps: step a writes thickness slot t of its index
    // (collectIntensity's t, stem3/stemlib.cpp:2597-2610); a slot keeps its
    // last writer only
    std::vector<int> lastWriter(nT, -1), slotOf(NS, -1);
    for (int a = 0; a < NS; a++) {
        const int x = stepIndex[a];
        const int t = (x < SA - 1) ? x / P.outputInterval : nT - 1;
        if (t < nT) lastWriter[t] = a;
    }
    for (int t = 0; t < nT; t++) if (lastWriter[t] >= 0) slotOf[lastWriter[t]] = t;
    const bool wantDet = ndet > 0 && det_images != nullptr;
    // QS_SERIES: one pattern / exit wave per thickness slot
    const bool series = (flags & QS_SERIES) != 0;
    const size_t nS = series ? (size_t)nT : 1;
    // QS_RESIDENT: the wave-resident loop (256 x 256, the band's columns
    // within the cluster's, no real-space waves of intermediate slots)
    int nbCols = 0;
    for (int iy = 0; iy < ny; iy++) nbCols += (iy <= yA || iy >= yB) ? 1 : 0;
    bool resident = (flags & QS_RESIDENT) && nx == 256 && ny == 256 && !(series && exit_waves) &&
                    nbCols <= resident_band_columns();
    if (resident) {
        int clusters = 0;
        QS_TRY(resident_clusters(&clusters));
        resident = clusters > 0;
    }
    // detector partial sums per wave: one per column tile, or one per CTA of
    // the resident loop's cluster
    const int detParts = resident ? 4 : ntiles;

    // device buffers: tables | tiles | positions
    void* dtab = nullptr;
    const size_t tabBytes = sizeof(float) * (nx + ny) + sizeof(float2) * (nx + ny);
    QS_TRY(ensure(c, B_TABLES, tabBytes, &dtab));
    float* d_kx2 = (float*)dtab;
    float* d_ky2 = d_kx2 + nx;
    float2* d_px = (float2*)(d_ky2 + ny);
    float2* d_py = d_px + nx;
    QS_CUDA_TRY(cudaMemcpyAsync(d_kx2, tb.kx2.data(), sizeof(float) * nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_ky2, tb.ky2.data(), sizeof(float) * ny, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_px, tb.px.data(), sizeof(float2) * nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_py, tb.py.data(), sizeof(float2) * ny, cudaMemcpyHostToDevice, s));
    void* dtiles = nullptr;
    QS_TRY(ensure(c, B_TILES, sizeof(int) * std::max(ntiles, 1), &dtiles));
    if (ntiles) QS_CUDA_TRY(cudaMemcpyAsync(dtiles, tiles.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, s));
    void* dpos = nullptr;
    QS_TRY(ensure(c, B_POS, sizeof(int) * 4 * (size_t)npos, &dpos));
    int* d_px_pos = (int*)dpos;
    int* d_py_pos = d_px_pos + npos;
    int* d_dx_pos = d_py_pos + npos;
    int* d_dy_pos = d_dx_pos + npos;
    QS_CUDA_TRY(cudaMemcpyAsync(d_px_pos, px.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_py_pos, py.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_dx_pos, dxp.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_dy_pos, dyp.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    int* d_steps = nullptr;  // resident loop: [stack slice | slot] of every step
    if (resident) {
        std::vector<int> st(stepSlice);
        st.insert(st.end(), slotOf.begin(), slotOf.end());
        void* d = nullptr;
        QS_TRY(ensure(c, B_STEPS, sizeof(int) * st.size(), &d));
        d_steps = (int*)d;
        QS_CUDA_TRY(cudaMemcpyAsync(d_steps, st.data(), sizeof(int) * st.size(), cudaMemcpyHostToDevice, s));
    }

    // transmission and probe
    const size_t nTrans = (size_t)S * P.potNx * P.potNy * (slabStacks ? D : 1);
    const float2* trans = (const float2*)trans_in;
    if (host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_TRANS, sizeof(float2) * nTrans, &d));
        QS_CUDA_TRY(cudaMemcpyAsync(d, trans_in, sizeof(float2) * nTrans, cudaMemcpyHostToDevice, s));
        trans = (const float2*)d;
    }
    void* dprobe = nullptr;
    if (probeStride) {
        dprobe = (void*)probe_in;
    } else if (probe_in) {
        QS_TRY(ensure(c, B_PROBE, sizeof(float2) * N, &dprobe));
        QS_CUDA_TRY(cudaMemcpyAsync(dprobe, probe_in, sizeof(float2) * N,
                                    host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
    } else {
        QS_TRY(ensure(c, B_PROBE, sizeof(float2) * N, &dprobe));
        QS_TRY(probe_into(c, P, (double)(nx / 2 * P.resolutionX), (double)(ny / 2 * P.resolutionY),
                          (float2*)dprobe));
    }

    // outputs
    float* det_dev = det_images;
    const size_t detElems = (size_t)nT * ndet * npix;
    if (wantDet && host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT1, sizeof(float) * detElems, &d));
        det_dev = (float*)d;
    }
    if (wantDet) QS_CUDA_TRY(cudaMemsetAsync(det_dev, 0, sizeof(float) * detElems, s));

    // batch chunking by free device memory (admission control)
    size_t freeB = 0, totalB = 0;
    QS_CUDA_TRY(cudaMemGetInfo(&freeB, &totalB));
    const size_t perWave = sizeof(float2) * N + (size_t)nT * detParts * std::max(ndet, 1) * sizeof(double) +
                           (host && diffpats ? sizeof(float) * N * nS : 0) +
                           (host && exit_waves ? sizeof(float2) * N * nS : 0);
    const size_t have = c->cap[B_WAVES] / (sizeof(float2) * N);
    const size_t budget = freeB > ((size_t)1 << 30) ? freeB - ((size_t)1 << 30) : freeB / 2;
    size_t chunk = std::min<size_t>((size_t)npos, std::max<size_t>(have, budget / perWave));
    if (chunk < 1) { set_error("not enough device memory for one wave"); return QS_ERR_NOMEM; }
    if (chunk < (size_t)npos) chunk = std::max<size_t>(1, chunk & ~(size_t)7);  // keep 8-row multiples

    void* dw = nullptr;
    QS_TRY(ensure(c, B_WAVES, sizeof(float2) * N * chunk, &dw));
    float2* waves = (float2*)dw;
    void* dpart = nullptr;
    const size_t partPerT = chunk * detParts * std::max(ndet, 1);
    QS_TRY(ensure(c, B_PARTIAL, sizeof(double) * partPerT * nT, &dpart));
    float* dp_dev = nullptr;
    if (diffpats && host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT2, sizeof(float) * N * chunk * nS, &d));
        dp_dev = (float*)d;
    }
    float2* ew_dev = nullptr;
    if (exit_waves && host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT3, sizeof(float2) * N * chunk * nS, &d));
        ew_dev = (float2*)d;
    }
    const float2* tw_y = twiddles(ny);
    const float2* tw_x = twiddles(nx, true);
    if (!tw_y || !tw_x) { set_error("twiddle table allocation failed"); return QS_ERR_NOMEM; }
    const double scaleDet = (double)P.electronScale / ((double)(nx * ny) * (double)(nx * ny));

    for (size_t p0 = 0; p0 < (size_t)npos; p0 += chunk) {
        const int nb = (int)std::min(chunk, (size_t)npos - p0);
        float* dpOut = diffpats ? (host ? dp_dev : diffpats + p0 * N) : nullptr;
        float2* ewOut = exit_waves ? (host ? ew_dev : (float2*)exit_waves + p0 * N) : nullptr;
        // distance between thickness slots of a series (elements)
        const size_t slotStride = N * (host ? chunk : (size_t)npos);

        RowArgs ra{};
        ra.nx = nx; ra.ny = ny; ra.potNx = P.potNx; ra.potNy = P.potNy;
        ra.nwaves = nb; ra.waves = waves; ra.exit_waves = nullptr;
        ra.probe = (const float2*)dprobe + p0 * probeStride;
        ra.probe_stride = probeStride;
        ra.trans_stride = transStride;
        const float2* transChunk = trans + p0 * transStride;
        ra.posX = d_px_pos + p0; ra.posY = d_py_pos + p0; ra.tw = tw_y; ra.yA = yA; ra.yB = yB;
        ra.norm = (float)(1.0 / (double)(nx * ny));
        ColArgs ca{};
        ca.nx = nx; ca.ny = ny; ca.nwaves = nb; ca.waves = waves; ca.tw = tw_x;
        ca.kx2 = d_kx2; ca.ky2 = d_ky2; ca.px = d_px; ca.py = d_py; ca.k2max = tb.k2max;
        ca.tiles = (const int*)dtiles; ca.ntiles = ntiles;
        for (int d = 0; d < ndet; d++) {
            ca.k2in[d] = P.detectors[d].k2Inside;
            ca.k2out[d] = P.detectors[d].k2Outside;
        }
        ca.scaleDiff = 1.0 / std::sqrt((double)(nx * ny));

        const double rowBytes = 24.0 * (double)N * nb, colBytes = 16.0 * (double)N * nb;
        auto rows = [&](RowMode m) -> int {
            size_t e0 = 0, e1 = 0;
            if (c->profile) QS_TRY(ev_record(c, &e0));
            QS_TRY(launch_rows(ra, m, s));
            if (c->profile) {
                QS_TRY(ev_record(c, &e1));
                c->row_ev.push_back({e0, e1});
                c->row_bytes += rowBytes;
            }
            return QS_OK;
        };
        auto cols = [&]() -> int {
            size_t e0 = 0, e1 = 0;
            if (c->profile) QS_TRY(ev_record(c, &e0));
            QS_TRY(launch_cols(ca, s));
            if (c->profile) {
                QS_TRY(ev_record(c, &e1));
                c->col_ev.push_back({e0, e1});
                c->col_bytes += colBytes;
            }
            return QS_OK;
        };
        // stack slice of step a
        auto sliceOf = [&](int a) { return transChunk + (size_t)stepSlice[a] * P.potNx * P.potNy; };
        // the chunk's stream work: the slice loop and the detector sums
        auto work = [&]() -> int {
        if (dpOut)
            for (size_t k = 0; k < nS; k++)
                QS_CUDA_TRY(cudaMemsetAsync(dpOut + k * slotStride, 0, sizeof(float) * N * nb, s));
        if (resident) {
            ResidentArgs r{};
            r.potNx = P.potNx; r.potNy = P.potNy; r.nwaves = nb; r.nsteps = NS;
            r.trans = transChunk; r.trans_stride = transStride;
            r.probe = ra.probe; r.probe_stride = probeStride;
            r.posX = ra.posX; r.posY = ra.posY;
            r.step_slice = d_steps; r.step_slot = d_steps + NS;
            r.tw = tw_y; r.yA = yA; r.yB = yB; r.nb = nbCols;
            r.kx2 = d_kx2; r.ky2 = d_ky2; r.px = d_px; r.py = d_py; r.k2max = tb.k2max;
            r.ndet = wantDet ? ndet : 0;
            for (int d = 0; d < ndet; d++) { r.k2in[d] = ca.k2in[d]; r.k2out[d] = ca.k2out[d]; }
            r.partial = (double*)dpart; r.partial_slot = partPerT;
            r.diffpat = dpOut; r.dp_slot = slotStride; r.series = series ? 1 : 0;
            r.exit_waves = ewOut; r.norm = ra.norm; r.scaleDiff = ca.scaleDiff;
            QS_TRY(launch_resident(r, s));
        } else {
        ra.trans_slice = sliceOf(0);
        QS_TRY(rows(ROW_FIRST));
        for (int a = 0; a < NS; a++) {
            const int slot = slotOf[a];
            ca.ndet = (wantDet && slot >= 0) ? ndet : 0;
            ca.partial = (double*)dpart + (slot >= 0 ? (size_t)slot * partPerT : 0);
            if (series)
                ca.diffpat = (dpOut && slot >= 0) ? dpOut + (size_t)slot * slotStride : nullptr;
            else
                ca.diffpat = (a == NS - 1) ? dpOut : nullptr;
            ca.inverse = (a < NS - 1 || ewOut) ? 1 : 0;
            QS_TRY(cols());
            if (series && ewOut && slot >= 0 && a < NS - 1) {
                // the real-space wave after step a, before the next transmit
                ra.exit_waves = ewOut + (size_t)slot * slotStride;
                QS_TRY(launch_rows(ra, ROW_LAST, s));
            }
            if (a < NS - 1) {
                ra.trans_slice = sliceOf(a + 1);
                QS_TRY(rows(ROW_MID));
            }
        }
        if (ewOut) {
            ra.exit_waves = ewOut + (series ? (size_t)(nT - 1) * slotStride : 0);
            QS_TRY(launch_rows(ra, ROW_LAST, s));
        }
        }
        if (wantDet)
            for (int t = 0; t < nT; t++) {
                if (lastWriter[t] < 0) continue;
                QS_TRY(launch_det_finalize((double*)dpart + (size_t)t * partPerT, nb, detParts, ndet, scaleDet,
                                           d_dx_pos + p0, d_dy_pos + p0, P.scanYN, npix,
                                           det_dev + (size_t)t * ndet * npix, s));
            }
        return QS_OK;
        };
        // QS_GRAPH (device buffers only): everything the launches bake in
        const bool graph = (flags & QS_GRAPH) && !host && !c->profile;
        KeyBytes key;
        if (graph)
            key.add(P).add(flags).add(trans_in).add(transStride).add(dprobe).add(probeStride).add(det_dev)
                .add(diffpats).add(exit_waves).add(p0).add(nb).add(chunk).add(npos).add(waves).add(dpart).add(dtab)
                .add(dtiles).add(dpos).add(tw_y).add(tw_x).add(d_steps);
        QS_TRY(run_graphed(c, s, graph, key.b, work));
        for (size_t k = 0; k < nS; k++) {
            if (host && diffpats)
                QS_CUDA_TRY(cudaMemcpyAsync(diffpats + (k * npos + p0) * N, dpOut + k * slotStride,
                                            sizeof(float) * N * nb, cudaMemcpyDeviceToHost, s));
            if (host && exit_waves)
                QS_CUDA_TRY(cudaMemcpyAsync(exit_waves + 2 * (k * npos + p0) * N, ewOut + k * slotStride,
                                            sizeof(float2) * N * nb, cudaMemcpyDeviceToHost, s));
        }
    }
    if (wantDet && host)
        QS_CUDA_TRY(cudaMemcpyAsync(det_images, det_dev, sizeof(float) * detElems, cudaMemcpyDeviceToHost, s));
    if (host || (flags & QS_SYNC)) QS_CUDA_TRY(cudaStreamSynchronize(s));
    return QS_OK;
}

int qs_multislice_run(qs_ctx* c, const qs_params* p, const float* trans_in, const float* probe_in,
                      const qs_batch* batch, float* det_images, float* diffpats, float* exit_waves, unsigned flags) {
    return multislice_run_ex(c, p, trans_in, 0, probe_in, 0, batch, det_images, diffpats, exit_waves, flags);
}

int qs_stem_run(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, const qs_batch* batch,
                float* det_images, float* diffpats) {
    if (!c || !batch) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    QS_CUDA_TRY(cudaSetDevice(c->device));
    const size_t nTrans = (size_t)p->slices * p->potNx * p->potNy;
    // doSTEM builds slab 0 once when the slabs are equal, else every slab
    // (stem3/stem3.cpp:2795-2812)
    const int nslab = (p->cellDiv > 1 && !p->equalDivs) ? p->cellDiv : 1;
    void* dstack = nullptr;
    // B_DIFF_IN doubles as the configuration's transmission stacks here
    QS_TRY(ensure(c, B_DIFF_IN, sizeof(float2) * nTrans * nslab, &dstack));
    for (int k = 0; k < nslab; k++)
        QS_TRY(qs_slab_build(c, p, atoms, natom, k, (float*)dstack + 2 * nTrans * k, 0));
    const qs_params& P = *p;
    const int nT = thickness_count(P);
    const int npix = P.scanXN * P.scanYN;
    const size_t N = (size_t)P.nx * P.ny;
    float* ddet = nullptr;
    float* ddp = nullptr;
    if (det_images && P.detectorNum > 0) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT1, sizeof(float) * (size_t)nT * P.detectorNum * npix, &d));
        ddet = (float*)d;
    }
    if (diffpats) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT2, sizeof(float) * N * batch->npos, &d));
        ddp = (float*)d;
    }
    // device buffers of the context throughout: repeated configurations of
    // one scan replay the slice loop as a CUDA graph
    QS_TRY(qs_multislice_run(c, p, (const float*)dstack, nullptr, batch, ddet, ddp, nullptr,
                             (nslab > 1 ? QS_SLAB_STACKS : 0) | QS_GRAPH));
    if (ddet)
        QS_CUDA_TRY(cudaMemcpyAsync(det_images, ddet, sizeof(float) * (size_t)nT * P.detectorNum * npix,
                                    cudaMemcpyDeviceToHost, c->stream));
    if (ddp)
        QS_CUDA_TRY(cudaMemcpyAsync(diffpats, ddp, sizeof(float) * N * batch->npos, cudaMemcpyDeviceToHost,
                                    c->stream));
    QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return QS_OK;
}

// ------------------------------------------------------------- CBED batch
namespace {

// Instances that share one batched scan: the same grid (the line transforms
// and launch shapes follow it).  Sampling, slice thickness, energy, optics,
// thickness, slabs and stacking sequence differ per wave: every wave carries
// its own propagator and k^2 tables, band, column-tile work items and
// step-to-slice table.
struct GridKey {
    int nx, ny, potNx, potNy;
    bool operator<(const GridKey& o) const {
        return std::tie(nx, ny, potNx, potNy) < std::tie(o.nx, o.ny, o.potNx, o.potNy);
    }
};

struct CbedUnit {
    std::vector<int> jobs;   // sorted by step count, descending
    int smax = 0;            // steps of the longest wave
    int kmax = 0;            // stack slices stored for the widest wave
    size_t bytes = 0;
};

size_t rup256(size_t b) { return (b + 255) & ~(size_t)255; }

// steps a wave takes: mulsRepeat2 passes through cellDiv slabs of `slices`,
// each slab's stack mulsRepeat1 times (doCBED's slab loop,
// stem3/stem3.cpp:2188-2219, around runMulsSTEM's repeat loop)
int abs_slices(const qs_params& P) {
    return P.slices * std::max(1, P.cellDiv) * std::max(1, P.mulsRepeat1) * std::max(1, P.mulsRepeat2);
}

// stack slices an instance stores: one stack per slab, slab 0's alone when
// the divisions are equal (the reference reuses it)
int stored_slices(const qs_params& P) {
    const int D = std::max(1, P.cellDiv);
    return P.slices * ((D > 1 && !P.equalDivs) ? D : 1);
}

// the stored slice each step transmits
void step_slices(const qs_params& P, std::vector<int>& out) {
    const int D = std::max(1, P.cellDiv), R1 = std::max(1, P.mulsRepeat1), R2 = std::max(1, P.mulsRepeat2);
    const bool perSlab = D > 1 && !P.equalDivs;
    out.clear();
    for (int pc = 0; pc < R2 * D; pc++)
        for (int r = 0; r < R1; r++)
            for (int i = 0; i < P.slices; i++) out.push_back((perSlab ? pc % D : 0) * P.slices + i);
}

// Device bytes of a unit of nb waves of one grid: stacks of kmax slices,
// probes, waves, patterns, per-wave tables, work items, step table.
size_t cbed_unit_bytes(const qs_params& P, int nb, int kmax, int smax) {
    const size_t N = (size_t)P.nx * P.ny, Pp = (size_t)P.potNx * P.potNy;
    const int C = col_tile_width(P.nx), tmax = (P.ny + C - 1) / C;
    return rup256(sizeof(float2) * Pp * kmax * nb) + 2 * rup256(sizeof(float2) * N * nb) +
           rup256(sizeof(float) * N * nb) + 2 * rup256(sizeof(float) * (size_t)(P.nx + P.ny) * nb) +
           2 * rup256(sizeof(float2) * (size_t)(P.nx + P.ny) * nb) + rup256(sizeof(float) * nb) +
           rup256(sizeof(int2) * nb) + rup256(sizeof(int2) * (size_t)nb * tmax) + rup256(sizeof(int) * (size_t)smax * nb) +
           rup256(sizeof(int) * nb);
}

}  // namespace

int qs_cbed_batch_run(qs_ctx* c, const qs_cbed_job* jobs, int njobs, size_t max_bytes, qs_cbed_report* rep) {
    if (!c || !jobs || njobs < 1) { set_error("null argument or no jobs"); return QS_ERR_ARG; }
    for (int i = 0; i < njobs; i++) {
        const qs_cbed_job& J = jobs[i];
        QS_TRY(check_params(&J.params));
        const qs_params& P = J.params;
        if (!J.diffpat || J.natom < 0 || (J.natom > 0 && !J.atoms)) {
            set_error("job " + std::to_string(i) + ": null output, atoms or negative atom count");
            return QS_ERR_ARG;
        }
        if (P.potNx != P.nx || P.potNy != P.ny) {
            set_error("job " + std::to_string(i) + ": CBED needs the potential grid equal to the wave grid");
            return QS_ERR_ARG;
        }
        if (!line_supported(P.nx) || !line_supported(P.ny)) {
            set_error("job " + std::to_string(i) + ": nx, ny must be in {64,128,256,384,512,768,1024}");
            return QS_ERR_UNSUPPORTED;
        }
    }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;

    // batches of instances of one grid, longest first inside each
    std::map<GridKey, std::vector<int>> groups;
    for (int i = 0; i < njobs; i++) {
        const qs_params& P = jobs[i].params;
        groups[GridKey{P.nx, P.ny, P.potNx, P.potNy}].push_back(i);
    }
    size_t freeB = 0, totalB = 0;
    QS_CUDA_TRY(cudaMemGetInfo(&freeB, &totalB));
    const size_t reserve = (size_t)1 << 30;
    size_t budget = freeB > reserve ? freeB - reserve : 0;
    if (max_bytes && max_bytes < budget) budget = max_bytes;
    // split each batch into units that fit the budget
    std::vector<CbedUnit> units;
    for (auto& g : groups) {
        std::vector<int>& v = g.second;
        std::stable_sort(v.begin(), v.end(),
                         [&](int a, int b) { return abs_slices(jobs[a].params) > abs_slices(jobs[b].params); });
        CbedUnit u;
        for (int i : v) {
            const qs_params& P = jobs[i].params;
            const int smax = u.jobs.empty() ? abs_slices(P) : u.smax;
            const int kmax = std::max(u.jobs.empty() ? 0 : u.kmax, stored_slices(P));
            if (!u.jobs.empty() && cbed_unit_bytes(P, (int)u.jobs.size() + 1, kmax, smax) > budget) {
                units.push_back(u);
                u = CbedUnit();
            }
            if (u.jobs.empty()) {
                u.smax = abs_slices(P);
                u.kmax = 0;
            }
            u.jobs.push_back(i);
            u.kmax = std::max(u.kmax, stored_slices(P));
            u.bytes = cbed_unit_bytes(P, (int)u.jobs.size(), u.kmax, u.smax);
            if (u.bytes > budget) {
                set_error("job " + std::to_string(i) + " needs " + std::to_string(u.bytes) +
                          " bytes of device memory, more than the " + std::to_string(budget) + " available");
                return QS_ERR_NOMEM;
            }
        }
        if (!u.jobs.empty()) units.push_back(u);
    }
    // rounds: first fit, largest unit first
    std::vector<int> order(units.size());
    for (size_t k = 0; k < order.size(); k++) order[k] = (int)k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return units[a].bytes > units[b].bytes; });
    std::vector<std::vector<int>> rounds;
    std::vector<size_t> roundBytes;
    for (int k : order) {
        size_t r = 0;
        while (r < rounds.size() && roundBytes[r] + units[k].bytes > budget) r++;
        if (r == rounds.size()) { rounds.emplace_back(); roundBytes.push_back(0); }
        rounds[r].push_back(k);
        roundBytes[r] += units[k].bytes;
    }
    const int nstreams = (int)std::min<size_t>(4, units.size());
    std::vector<cudaStream_t> streams(nstreams, nullptr);
    std::vector<cudaEvent_t> evs(nstreams, nullptr);
    auto cleanup = [&]() {
        for (auto& e : evs) if (e) cudaEventDestroy(e);
        for (auto& t : streams) if (t) cudaStreamDestroy(t);
    };
    int rc = QS_OK;
    for (int k = 0; k < nstreams && rc == QS_OK; k++) {
        if (cudaStreamCreateWithFlags(&streams[k], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&evs[k], cudaEventDisableTiming) != cudaSuccess) {
            set_error("stream or event creation failed");
            rc = QS_ERR_CUDA;
        }
    }
    size_t admitted = 0;
    for (size_t r = 0; r < rounds.size() && rc == QS_OK; r++) {
        rc = [&]() -> int {
            void* base = nullptr;
            QS_TRY(ensure(c, B_CBED, roundBytes[r], &base));
            admitted = std::max(admitted, roundBytes[r]);
            unsigned char* cur = (unsigned char*)base;
            auto take = [&](size_t b) { void* q = cur; cur += rup256(b); return q; };
            struct Carved {
                float2 *stacks, *probes, *waves;
                float* dp;
                float *kx2, *ky2, *k2max;
                float2 *px, *py;
                int2 *band, *items;
                int *steps, *zeros;
                std::vector<int> itemStart;  // first work item of each wave (+ the total)
                std::vector<int> S;          // steps of each wave
            };
            std::vector<Carved> cv(rounds[r].size());
            // host copies of the round's tables, alive until the round's
            // closing synchronisation
            std::vector<std::vector<unsigned char>> hostTabs(rounds[r].size());
            // one event per unit, recorded once its stacks and probes are
            // built: its scan starts then, while later units still build
            std::vector<cudaEvent_t> built(rounds[r].size(), nullptr);
            struct EvGuard {
                std::vector<cudaEvent_t>& v;
                ~EvGuard() { for (auto e : v) if (e) cudaEventDestroy(e); }
            } guard{built};
            for (auto& e : built) QS_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            // 1. slice stacks, probes and per-wave tables on the context's stream
            for (size_t k = 0; k < rounds[r].size(); k++) {
                const CbedUnit& u = units[rounds[r][k]];
                const qs_params& P0 = jobs[u.jobs[0]].params;
                const int nb = (int)u.jobs.size(), nx = P0.nx, ny = P0.ny;
                const size_t N = (size_t)nx * ny, Pp = (size_t)P0.potNx * P0.potNy;
                const int Cw = col_tile_width(nx), tmax = (ny + Cw - 1) / Cw;
                Carved& C = cv[k];
                C.stacks = (float2*)take(sizeof(float2) * Pp * u.kmax * nb);
                C.probes = (float2*)take(sizeof(float2) * N * nb);
                C.waves = (float2*)take(sizeof(float2) * N * nb);
                C.dp = (float*)take(sizeof(float) * N * nb);
                C.kx2 = (float*)take(sizeof(float) * (size_t)nx * nb);
                C.ky2 = (float*)take(sizeof(float) * (size_t)ny * nb);
                C.px = (float2*)take(sizeof(float2) * (size_t)nx * nb);
                C.py = (float2*)take(sizeof(float2) * (size_t)ny * nb);
                C.k2max = (float*)take(sizeof(float) * nb);
                C.band = (int2*)take(sizeof(int2) * nb);
                C.items = (int2*)take(sizeof(int2) * (size_t)nb * tmax);
                C.steps = (int*)take(sizeof(int) * (size_t)u.smax * nb);
                C.zeros = (int*)take(sizeof(int) * nb);
                // host side: tables, bands, work items (grouped by wave) and
                // the step-to-slice table [step][wave]
                std::vector<float> kx2(nx * (size_t)nb), ky2(ny * (size_t)nb), k2m(nb);
                std::vector<float2> pxv(nx * (size_t)nb), pyv(ny * (size_t)nb);
                std::vector<int2> band(nb), items;
                std::vector<int> steps((size_t)u.smax * nb, 0), st;
                C.S.resize(nb);
                C.itemStart.assign(nb + 1, 0);
                for (int w = 0; w < nb; w++) {
                    const qs_params& P = jobs[u.jobs[w]].params;
                    const PropTables tb = prop_tables(P);
                    const Band bd = band_tiles(tb, ny, Cw);
                    std::copy(tb.kx2.begin(), tb.kx2.end(), kx2.begin() + (size_t)w * nx);
                    std::copy(tb.ky2.begin(), tb.ky2.end(), ky2.begin() + (size_t)w * ny);
                    std::copy(tb.px.begin(), tb.px.end(), pxv.begin() + (size_t)w * nx);
                    std::copy(tb.py.begin(), tb.py.end(), pyv.begin() + (size_t)w * ny);
                    k2m[w] = tb.k2max;
                    band[w] = make_int2(bd.yA, bd.yB);
                    C.itemStart[w] = (int)items.size();
                    for (int t0 : bd.tiles) items.push_back(make_int2(w, t0));
                    step_slices(P, st);
                    C.S[w] = (int)st.size();
                    for (size_t a = 0; a < st.size(); a++) steps[a * nb + w] = st[a];
                }
                C.itemStart[nb] = (int)items.size();
                // one host block per unit (kept in hostTabs), copied piece by piece
                std::vector<unsigned char>& H = hostTabs[k];
                struct Up { void* dst; size_t off, bytes; };
                std::vector<Up> ups;
                auto add = [&](void* dst, const void* src, size_t bytes) {
                    if (!bytes) return;
                    const size_t off = H.size();
                    H.resize(off + bytes);
                    std::memcpy(H.data() + off, src, bytes);
                    ups.push_back({dst, off, bytes});
                };
                add(C.kx2, kx2.data(), sizeof(float) * kx2.size());
                add(C.ky2, ky2.data(), sizeof(float) * ky2.size());
                add(C.px, pxv.data(), sizeof(float2) * pxv.size());
                add(C.py, pyv.data(), sizeof(float2) * pyv.size());
                add(C.k2max, k2m.data(), sizeof(float) * k2m.size());
                add(C.band, band.data(), sizeof(int2) * band.size());
                add(C.items, items.data(), sizeof(int2) * items.size());
                add(C.steps, steps.data(), sizeof(int) * steps.size());
                for (const Up& up : ups)
                    QS_CUDA_TRY(cudaMemcpyAsync(up.dst, H.data() + up.off, up.bytes, cudaMemcpyHostToDevice, s));
                QS_CUDA_TRY(cudaMemsetAsync(C.zeros, 0, sizeof(int) * nb, s));
                QS_CUDA_TRY(cudaMemsetAsync(C.dp, 0, sizeof(float) * N * nb, s));
                for (int w = 0; w < nb; w++) {
                    const qs_cbed_job& J = jobs[u.jobs[w]];
                    // one stack per slab (slab 0's alone for equal divisions)
                    float2* st0 = C.stacks + (size_t)w * u.kmax * Pp;
                    const int nslab = stored_slices(J.params) / J.params.slices;
                    for (int slab = 0; slab < nslab; slab++)
                        QS_TRY(qs_slab_build(c, &J.params, J.atoms, J.natom, slab,
                                             (float*)(st0 + (size_t)slab * J.params.slices * Pp), 0));
                    // doCBED's probe position (stem3/stem3.cpp:2096-2100)
                    const double dx = (double)(J.params.scanXStart - J.params.potOffsetX);
                    const double dy = (double)(J.params.scanYStart - J.params.potOffsetY);
                    QS_TRY(probe_into(c, J.params, dx, dy, C.probes + (size_t)w * N));
                }
                if (!twiddles(nx, true) || !twiddles(ny)) { set_error("twiddle table allocation failed"); return QS_ERR_NOMEM; }
                QS_CUDA_TRY(cudaEventRecord(built[k], s));
            }
            // 2. the units' scans, concurrently on the side streams, each
            // after its own unit's build: per step
            // one row pass over the waves still running and one column pass
            // for those that go on (inverse) or end here (pattern)
            for (size_t k = 0; k < rounds[r].size(); k++) {
                const CbedUnit& u = units[rounds[r][k]];
                const Carved& C = cv[k];
                cudaStream_t st = streams[k % nstreams];
                QS_CUDA_TRY(cudaStreamWaitEvent(st, built[k], 0));
                const qs_params& P0 = jobs[u.jobs[0]].params;
                const int nb = (int)u.jobs.size(), nx = P0.nx, ny = P0.ny;
                const size_t N = (size_t)nx * ny, Pp = (size_t)P0.potNx * P0.potNy;
                RowArgs ra{};
                ra.nx = nx; ra.ny = ny; ra.potNx = P0.potNx; ra.potNy = P0.potNy;
                ra.probe = C.probes; ra.probe_stride = N; ra.trans_stride = (size_t)u.kmax * Pp;
                ra.trans_slice = C.stacks; ra.band = C.band;
                ra.waves = C.waves; ra.posX = C.zeros; ra.posY = C.zeros; ra.tw = twiddles(ny);
                ra.norm = (float)(1.0 / (double)N);
                ColArgs ca{};
                ca.nx = nx; ca.ny = ny; ca.tw = twiddles(nx, true); ca.kx2 = C.kx2; ca.ky2 = C.ky2; ca.px = C.px;
                ca.py = C.py; ca.per_wave = 1; ca.k2max_w = C.k2max; ca.waves = C.waves; ca.ndet = 0;
                ca.scaleDiff = 1.0 / std::sqrt((double)N);
                for (int sl = 0; sl < u.smax; sl++) {
                    int active = 0, cont = 0;
                    for (int w = 0; w < nb; w++) {
                        active += C.S[w] > sl;
                        cont += C.S[w] > sl + 1;
                    }
                    ra.nwaves = active;
                    ra.step_slice = C.steps + (size_t)sl * nb;
                    QS_TRY(launch_rows(ra, sl == 0 ? ROW_FIRST : ROW_MID, st));
                    if (cont > 0) {
                        ca.nwaves = cont; ca.items = C.items; ca.nitems = C.itemStart[cont];
                        ca.inverse = 1; ca.diffpat = nullptr;
                        QS_TRY(launch_cols(ca, st));
                    }
                    if (active > cont) {
                        // waves whose last step this is: the pattern, no inverse
                        ca.nwaves = active; ca.items = C.items + C.itemStart[cont];
                        ca.nitems = C.itemStart[active] - C.itemStart[cont];
                        ca.inverse = 0; ca.diffpat = C.dp;
                        QS_TRY(launch_cols(ca, st));
                    }
                }
                QS_CUDA_TRY(cudaEventRecord(evs[k % nstreams], st));
                QS_CUDA_TRY(cudaStreamWaitEvent(s, evs[k % nstreams], 0));
            }
            // 3. patterns back to the host
            for (size_t k = 0; k < rounds[r].size(); k++) {
                const CbedUnit& u = units[rounds[r][k]];
                const size_t N = (size_t)jobs[u.jobs[0]].params.nx * jobs[u.jobs[0]].params.ny;
                for (size_t w = 0; w < u.jobs.size(); w++)
                    QS_CUDA_TRY(cudaMemcpyAsync(jobs[u.jobs[w]].diffpat, cv[k].dp + w * N, sizeof(float) * N,
                                                cudaMemcpyDeviceToHost, s));
            }
            QS_CUDA_TRY(cudaStreamSynchronize(s));
            return QS_OK;
        }();
    }
    if (rc != QS_OK) {
        // leave no side-stream work in flight
        for (auto& t : streams) if (t) cudaStreamSynchronize(t);
        cudaStreamSynchronize(s);
    }
    cleanup();
    if (rc == QS_OK && rep) {
        rep->groups = (int)groups.size();
        rep->rounds = (int)rounds.size();
        rep->streams = nstreams;
        rep->admitted_bytes = (double)admitted;
        rep->budget_bytes = (double)budget;
    }
    return rc;
}

int qs_tem_run(qs_ctx* c, const qs_params* p, const qs_atom* atoms, const int* natoms, int nconf, const qs_ctf* ctf,
               int ndef, const double* defoci, float* mean_intensity, float* ctf_images, float* exit_waves) {
    return qs_tem_run_tilted(c, p, 0.0, 0.0, atoms, natoms, nconf, ctf, ndef, defoci, mean_intensity, ctf_images,
                             exit_waves);
}

int qs_tem_run_tilted(qs_ctx* c, const qs_params* p, double btiltx, double btilty, const qs_atom* atoms,
                      const int* natoms, int nconf, const qs_ctf* ctf, int ndef, const double* defoci,
                      float* mean_intensity, float* ctf_images, float* exit_waves) {
    if (!c || !natoms || nconf < 1) { set_error("null argument or no configurations"); return QS_ERR_ARG; }
    if (ndef > 0 && ctf_images && (!ctf || !defoci)) { set_error("CTF images need ctf and defoci"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    const qs_params& P = *p;
    QS_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const int nx = P.nx, ny = P.ny;
    const size_t N = (size_t)nx * ny;
    // a cell divided into slabs: one stack per slab unless they are equal
    // (doTEM's slab loop, stem3/stem3.cpp:2473-2537)
    const int nslab = (P.cellDiv > 1 && !P.equalDivs) ? P.cellDiv : 1;
    const size_t slabStack = (size_t)P.slices * P.potNx * P.potNy;
    const size_t stack = slabStack * nslab;
    const int nimg = (ctf_images && ndef > 0) ? ndef : 0;
    size_t natomTotal = 0;
    for (int k = 0; k < nconf; k++) {
        if (natoms[k] < 0) { set_error("negative atom count"); return QS_ERR_ARG; }
        natomTotal += (size_t)natoms[k];
    }
    if (natomTotal > 0 && !atoms) { set_error("null atoms"); return QS_ERR_ARG; }

    // configurations per batch: stack + exit wave + k-space copy + scratch +
    // the scan's own wave buffer, within the free memory less 1 GiB
    size_t freeB = 0, totalB = 0;
    QS_CUDA_TRY(cudaMemGetInfo(&freeB, &totalB));
    const size_t perConf = sizeof(float2) * (stack + (nimg ? 4 : 2) * N);
    const size_t fixed = sizeof(float2) * N * (1 + nimg) + sizeof(float) * N * (1 + nimg);
    const size_t budget = freeB > ((size_t)1 << 30) + fixed ? freeB - ((size_t)1 << 30) - fixed : 0;
    const int chunk = (int)std::min<size_t>((size_t)nconf, budget / perConf);
    if (chunk < 1) { set_error("not enough device memory for one configuration"); return QS_ERR_NOMEM; }

    // carve: stacks | exit waves | k-space | scratch | plane wave | H | accumulators
    auto rup = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t waveB = sizeof(float2) * N;
    const size_t total = rup(sizeof(float2) * stack * chunk) + rup(waveB * chunk) * (nimg ? 3 : 1) + rup(waveB) +
                         rup(waveB) + rup(sizeof(float) * N * (1 + nimg));
    void* base = nullptr;
    QS_TRY(ensure(c, B_TEM, total, &base));
    unsigned char* cur = (unsigned char*)base;
    auto take = [&](size_t b) { void* q = cur; cur += rup(b); return q; };
    float2* stacks = (float2*)take(sizeof(float2) * stack * chunk);
    float2* ew = (float2*)take(waveB * chunk);
    float2* kw = nimg ? (float2*)take(waveB * chunk) : nullptr;
    float2* scr = nimg ? (float2*)take(waveB * chunk) : nullptr;
    float2* plane = (float2*)take(waveB);
    float2* H = (float2*)take(waveB);
    float* acc = (float*)take(sizeof(float) * N * (1 + nimg));
    QS_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(float) * N * (1 + nimg), s));
    // doTEM's incident wave without beam tilt (stem3/stem3.cpp:2403-2406)
    QS_TRY(launch_fill(plane, N, 1.f, 0.f, s));
    std::vector<float2> tilted;
    if (btiltx != 0.0 || btilty != 0.0) {
        // doTEM's tilted plane wave (stem3/stem3.cpp:2409-2419): phase
        // k_t.(x, y) with k_t = 2 pi sin(tilt) / lambda in double, x =
        // dx (ix - nx/2) in float, and y formed from ix as the reference forms
        // it, so every row ix is constant along y
        const double pi = 3.1415926535897;
        const double lam = wavelength(P.v0);
        const double ktx = 2.0 * pi * std::sin((double)(float)btiltx) / lam;
        const double kty = 2.0 * pi * std::sin((double)(float)btilty) / lam;
        tilted.resize(N);
        for (int ix = 0; ix < nx; ix++) {
            const double x = (double)(P.resolutionX * (float)(ix - nx / 2));
            const double y = (double)(P.resolutionY * (float)(ix - nx / 2));
            const float2 v = make_float2((float)std::cos(ktx * x + kty * y), (float)std::sin(ktx * x + kty * y));
            for (int iy = 0; iy < ny; iy++) tilted[(size_t)ix * ny + iy] = v;
        }
        QS_CUDA_TRY(cudaMemcpyAsync(plane, tilted.data(), waveB, cudaMemcpyHostToDevice, s));
    }

    const double lambda = wavelength(P.v0);
    const float inv = 1.0f / (float)nconf;
    const float invImg = (float)(1.0 / ((double)nconf * (double)N * (double)N));
    std::vector<int> zeros(chunk, 0);
    size_t atomOff = 0;
    for (int c0 = 0; c0 < nconf; c0 += chunk) {
        const int nb = std::min(chunk, nconf - c0);
        for (int k = 0; k < nb; k++) {
            for (int slab = 0; slab < nslab; slab++)
                QS_TRY(qs_slab_build(c, p, atoms ? atoms + atomOff : nullptr, natoms[c0 + k], slab,
                                     (float*)(stacks + (size_t)k * stack + (size_t)slab * slabStack), 0));
            atomOff += (size_t)natoms[c0 + k];
        }
        qs_batch bt{nb, zeros.data(), zeros.data(), zeros.data(), zeros.data()};
        QS_TRY(multislice_run_ex(c, p, (const float*)stacks, stack, (const float*)plane, 0, &bt, nullptr, nullptr,
                                 (float*)ew, nslab > 1 ? QS_SLAB_STACKS : 0));
        QS_TRY(launch_acc_intensity(ew, nb, N, inv, acc, s));
        if (exit_waves)
            QS_CUDA_TRY(cudaMemcpyAsync(exit_waves + 2 * (size_t)c0 * N, ew, waveB * nb, cudaMemcpyDeviceToHost, s));
        if (nimg) {
            // FFT(psi) once, then per defocus IFFT(FFT(psi) H) and |.|^2
            QS_CUDA_TRY(cudaMemcpyAsync(kw, ew, waveB * nb, cudaMemcpyDeviceToDevice, s));
            QS_TRY(fft2d(kw, nx, ny, nb, false, s));
            for (int d = 0; d < nimg; d++) {
                QS_TRY(launch_ctf_table(nx, ny, P.resolutionX, P.resolutionY, lambda, *ctf, defoci[d], H, s));
                QS_TRY(launch_mul_table(kw, H, nb, N, scr, s));
                QS_TRY(fft2d(scr, nx, ny, nb, true, s));
                QS_TRY(launch_acc_intensity(scr, nb, N, invImg, acc + (size_t)(1 + d) * N, s));
            }
        }
    }
    if (mean_intensity)
        QS_CUDA_TRY(cudaMemcpyAsync(mean_intensity, acc, sizeof(float) * N, cudaMemcpyDeviceToHost, s));
    if (nimg)
        QS_CUDA_TRY(cudaMemcpyAsync(ctf_images, acc + N, sizeof(float) * N * nimg, cudaMemcpyDeviceToHost, s));
    QS_CUDA_TRY(cudaStreamSynchronize(s));
    return QS_OK;
}

int qs_phase_grating(qs_ctx* c, const qs_params* p, const float* V, float* trans, unsigned flags) {
    if (!c || !V || !trans) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    if (p->bandlimittrans) {
        set_error("qs_phase_grating: use qs_slices_build for band-limited transmission functions");
        return QS_ERR_UNSUPPORTED;
    }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    const size_t n = (size_t)p->slices * p->potNx * p->potNy;
    const double mm0 = (double)(1.0f + p->v0 / 511.0f);
    QS_TRY(launch_grating_from_real(V, (float2*)trans, n, mm0 * wavelength(p->v0), c->stream));
    if (flags & QS_SYNC) QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return QS_OK;
}

int qs_adjoint_run(qs_ctx* c, const qs_params* p, const float* trans_in, const float* probe_in,
                   const qs_batch* batch, const float* target, int ckpt, double* loss, float* dL_dV, float* diffpats,
                   unsigned flags) {
    if (!c || !trans_in || !probe_in || !batch || !target || !dL_dV) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    const qs_params& P = *p;
    if (!line_supported(P.nx) || !line_supported(P.ny)) {
        set_error("adjoint: nx, ny must be in {64,128,256,384,512,768,1024}");
        return QS_ERR_UNSUPPORTED;
    }
    if (P.bandlimittrans) {
        set_error("adjoint: band-limited transmission functions are not supported");
        return QS_ERR_UNSUPPORTED;
    }
    // the steps: mulsRepeat2 passes through cellDiv slabs of `slices`, each
    // slab's stack mulsRepeat1 times (doSTEM's slab loop around runMulsSTEM's
    // repeats); the stack is one per slab with QS_SLAB_STACKS, else one
    // reused.  Step a transmits stack slice stepStack[a]; a stack slice's
    // dL/dV sums the gradients of all its steps.
    const int npos = batch->npos, S0 = P.slices, D = std::max(1, P.cellDiv), nx = P.nx, ny = P.ny;
    const bool slabStacks = D > 1 && (flags & QS_SLAB_STACKS);
    std::vector<int> stepStack;
    for (int pc = 0; pc < std::max(1, P.mulsRepeat2) * D; pc++)
        for (int r = 0; r < std::max(1, P.mulsRepeat1); r++)
            for (int i = 0; i < S0; i++) stepStack.push_back((slabStacks ? (pc % D) * S0 : 0) + i);
    const int S = (int)stepStack.size();
    std::vector<int> lastUse(slabStacks ? D * S0 : S0, -1);
    for (int a = 0; a < S; a++) lastUse[stepStack[a]] = a;
    auto stackIdx = [&](int a) { return stepStack[a]; };
    if (npos < 1) { set_error("batch has no positions"); return QS_ERR_ARG; }
    QS_TRY(check_raster(P, *batch, false));
    if (ckpt < 1) {
        // automatic: every state kept when they fit (no recomputation), else
        // the smallest interval whose checkpoints and segment states fit
        size_t freeB = 0, totalB = 0;
        QS_CUDA_TRY(cudaMemGetInfo(&freeB, &totalB));
        const size_t reserve = (size_t)1 << 30;
        const size_t budget = freeB > reserve ? freeB - reserve : 0;
        const size_t wave = sizeof(float2) * (size_t)nx * ny * npos;
        ckpt = S;
        for (int k = 1; k < S; k++) {
            const size_t nbufs = 4 + (size_t)((S + k - 1) / k - 1) + (size_t)(k - 1);
            if (nbufs * wave <= budget) { ckpt = k; break; }
        }
    }
    if (ckpt > S) ckpt = S;
    QS_CUDA_TRY(cudaSetDevice(c->device));
    cudaStream_t s = c->stream;
    const size_t N = (size_t)nx * ny;

    std::vector<int> px(npos), py(npos);
    for (int i = 0; i < npos; i++) {
        if (batch->iPosX && batch->iPosY) {
            px[i] = batch->iPosX[i];
            py[i] = batch->iPosY[i];
        } else {
            const int ix = i / P.scanYN, iy = i % P.scanYN;
            int x = (int)((float)ix * (P.scanXStop - P.scanXStart) / ((float)P.scanXN * P.resolutionX));
            int y = (int)((float)iy * (P.scanYStop - P.scanYStart) / ((float)P.scanYN * P.resolutionY));
            px[i] = std::min(x, P.potNx - nx);
            py[i] = std::min(y, P.potNy - ny);
        }
        if (px[i] < 0 || py[i] < 0 || px[i] > P.potNx - nx || py[i] > P.potNy - ny) {
            set_error("position " + std::to_string(i) + " puts the window outside the potential array");
            return QS_ERR_ARG;
        }
    }
    PropTables tb = prop_tables(P);
    const int C = col_tile_width(nx);
    const Band band = band_tiles(tb, ny, C);
    const int yA = band.yA, yB = band.yB;
    const std::vector<int>& tiles = band.tiles;
    const int ntiles = (int)tiles.size();
    std::vector<float2> pxc(tb.px), pyc(tb.py);
    for (auto& v : pxc) v.y = -v.y;
    for (auto& v : pyc) v.y = -v.y;

    // device memory: tables | tiles | positions | loss partials | buffers
    const int nseg = (S + ckpt - 1) / ckpt;
    const size_t waveBytes = sizeof(float2) * N * npos;
    const size_t nLoss = (size_t)npos * (ny / C);
    auto rup = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t small = rup(sizeof(float) * (nx + ny)) + 2 * rup(sizeof(float2) * (nx + ny)) +
                         rup(sizeof(int) * std::max(ntiles, 1)) + rup(sizeof(int) * 2 * npos) + rup(sizeof(double) * nLoss);
    // dL/dV summed over positions with float atomics into one L2-resident
    // window sum per slice, or (QS_DETERMINISTIC) every position's g_t kept
    // and gathered in a fixed order
    const bool det = (flags & QS_DETERMINISTIC) != 0;
    // work, scratch state, grad, [grad_t], checkpoints 1..nseg-1, segment states 1..ckpt-1
    const size_t nbuf = (det ? 4 : 3) + (size_t)(nseg - 1) + (size_t)(ckpt - 1);
    const size_t partBytes = det ? dv_partial_bytes(npos, P.potNx, P.potNy)
                                 : sizeof(float2) * (size_t)P.potNx * P.potNy;
    void* base = nullptr;
    QS_TRY(ensure(c, B_ADJ, small + rup(partBytes) + nbuf * rup(waveBytes), &base));
    unsigned char* cur = (unsigned char*)base;
    auto take = [&](size_t b) { void* q = cur; cur += rup(b); return q; };
    float* d_kx2 = (float*)take(sizeof(float) * (nx + ny));
    float* d_ky2 = d_kx2 + nx;
    float2* d_px = (float2*)take(sizeof(float2) * (nx + ny));
    float2* d_py = d_px + nx;
    float2* d_pxc = (float2*)take(sizeof(float2) * (nx + ny));
    float2* d_pyc = d_pxc + nx;
    int* d_tiles = (int*)take(sizeof(int) * std::max(ntiles, 1));
    int* d_pos = (int*)take(sizeof(int) * 2 * npos);
    double* d_loss = (double*)take(sizeof(double) * nLoss);
    void* d_part = take(partBytes);
    float2* work = (float2*)take(waveBytes);
    float2* hscr = (float2*)take(waveBytes);
    float2* grad = (float2*)take(waveBytes);
    float2* grad_t = det ? (float2*)take(waveBytes) : nullptr;
    std::vector<float2*> ck(nseg, nullptr), seg(ckpt, nullptr);
    for (int k = 1; k < nseg; k++) ck[k] = (float2*)take(waveBytes);
    for (int k = 1; k < ckpt; k++) seg[k] = (float2*)take(waveBytes);

    QS_CUDA_TRY(cudaMemcpyAsync(d_kx2, tb.kx2.data(), sizeof(float) * nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_ky2, tb.ky2.data(), sizeof(float) * ny, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_px, tb.px.data(), sizeof(float2) * nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_py, tb.py.data(), sizeof(float2) * ny, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_pxc, pxc.data(), sizeof(float2) * nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_pyc, pyc.data(), sizeof(float2) * ny, cudaMemcpyHostToDevice, s));
    if (ntiles) QS_CUDA_TRY(cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_pos, px.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync(d_pos + npos, py.data(), sizeof(int) * npos, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemsetAsync(work, 0, waveBytes, s));
    QS_CUDA_TRY(cudaMemsetAsync(hscr, 0, waveBytes, s));
    QS_CUDA_TRY(cudaMemsetAsync(grad, 0, waveBytes, s));
    if (!det) QS_CUDA_TRY(cudaMemsetAsync(d_part, 0, partBytes, s));  // the window sum starts at zero
    const float2* tw_y = twiddles(ny);
    const float2* tw_x = twiddles(nx, true);
    if (!tw_y || !tw_x) { set_error("twiddle table allocation failed"); return QS_ERR_NOMEM; }
    const float2* trans = (const float2*)trans_in;
    const float2* probe = (const float2*)probe_in;
    const size_t sliceElems = (size_t)P.potNx * P.potNy;

    RowArgs ra{};
    ra.nx = nx; ra.ny = ny; ra.potNx = P.potNx; ra.potNy = P.potNy; ra.nwaves = npos; ra.probe = probe;
    ra.posX = d_pos; ra.posY = d_pos + npos; ra.tw = tw_y; ra.yA = yA; ra.yB = yB;
    ra.norm = (float)(1.0 / (double)N);
    ColArgs ca{};
    ca.nx = nx; ca.ny = ny; ca.nwaves = npos; ca.tw = tw_x; ca.kx2 = d_kx2; ca.ky2 = d_ky2;
    ca.k2max = tb.k2max; ca.tiles = d_tiles; ca.ntiles = ntiles; ca.inverse = 1; ca.ndet = 0;
    // Segments of ckpt slices, the remainder of S/ckpt first: segment k
    // starts at segStart[k] (checkpoints every ckpt slices counted back from
    // the end), so the segment the full run keeps whole -- the last, never
    // recomputed -- is a full one and the short one is recomputed instead.
    std::vector<int> segStart(nseg + 1, 0), ckOf(S + 1, -1);
    for (int k = 1; k < nseg; k++) segStart[k] = S - (nseg - k) * ckpt;
    segStart[nseg] = S;
    for (int k = 1; k < nseg; k++) ckOf[segStart[k]] = k;
    // Forward through slices [s0, upto).  The row pass of slice s reads the
    // state h_s (the probe for s = 0) and writes `work`; the column pass reads
    // `work` and writes h_{s+1} straight into the buffer that keeps it, so no
    // state is ever copied.  The full run (full true) keeps the checkpoint
    // states h_{segStart[k]} in ck[k] and the states of the last segment in
    // seg, and ends after the last row pass (the last column pass is the loss
    // kernel).  A segment recompute writes h_s, s0 < s < upto, into seg.
    const int lastS0 = segStart[nseg - 1];
    auto state_of = [&](int sl, int s0) -> float2* {
        if (sl == 0) return nullptr;
        if (sl > s0) return seg[sl - s0];
        return ck[ckOf[sl]];
    };
    auto forward = [&](int s0, int upto, bool full) -> int {
        ca.px = d_px;
        ca.py = d_py;
        const int last = full ? upto : upto - 1;
        float2* cur = state_of(s0, s0);
        for (int sl = s0; sl < last; sl++) {
            ra.waves = cur;
            ra.waves_out = work;
            ra.trans_slice = trans + (size_t)stackIdx(sl) * sliceElems;
            QS_TRY(launch_rows(ra, sl == 0 ? ROW_FIRST : ROW_MID, s));
            if (sl == S - 1) break;
            const int nxt = sl + 1;
            float2* dst;
            if (!full || nxt > lastS0) dst = seg[nxt - (full ? lastS0 : s0)];
            else if (ckOf[nxt] >= 0) dst = ck[ckOf[nxt]];
            else dst = hscr;
            ca.waves = work;
            ca.waves_out = dst;
            QS_TRY(launch_cols(ca, s));
            cur = dst;
        }
        return QS_OK;
    };
    // 1. forward through all slices
    QS_TRY(forward(0, S, true));
    // 2. loss and its gradient at the last slice: g_A of slice S-1 in `grad`
    AdjLastArgs la{};
    la.nx = nx; la.ny = ny; la.nwaves = npos; la.yA = yA; la.yB = yB; la.waves = work; la.waves_out = grad;
    la.tw = tw_x;
    la.kx2 = d_kx2; la.ky2 = d_ky2; la.px = d_px; la.py = d_py; la.k2max = tb.k2max; la.target = target;
    la.diffpat = diffpats; la.scaleDiff = 1.0 / std::sqrt((double)N); la.loss_partial = d_loss;
    QS_TRY(launch_adj_last(la, s));
    // 3. backward, segment by segment
    const double sigma = (double)(1.0f + P.v0 / 511.0f) * wavelength(P.v0);
    AdjRowArgs ar{};
    ar.nx = nx; ar.ny = ny; ar.potNx = P.potNx; ar.potNy = P.potNy; ar.nwaves = npos; ar.yA = yA; ar.yB = yB;
    ar.grad = grad; ar.probe = probe; ar.grad_t = grad_t; ar.gsum = det ? nullptr : (float2*)d_part;
    ar.posX = d_pos; ar.posY = d_pos + npos; ar.tw = tw_y;
    ar.norm = (float)(1.0 / (double)N);
    for (int sg = nseg - 1; sg >= 0; sg--) {
        const int s0 = segStart[sg], s1 = segStart[sg + 1];
        // recompute the segment's states h_s, s0 < s < s1 (the full run kept
        // those of the last segment)
        if (sg < nseg - 1 && s1 - s0 > 1) QS_TRY(forward(s0, s1, false));
        for (int sl = s1 - 1; sl >= s0; sl--) {
            if (sl < S - 1) {
                // column pass with conj(P): g_h(sl+1) -> g_A(sl)
                ca.waves = grad;
                ca.waves_out = nullptr;
                ca.px = d_pxc;
                ca.py = d_pyc;
                QS_TRY(launch_cols(ca, s));
            }
            ar.state = state_of(sl, s0);
            ar.trans_slice = trans + (size_t)stackIdx(sl) * sliceElems;
            QS_TRY(launch_adj_rows(ar, sl == 0, s));
            // a reused stack's slice collects the gradient of every use; the
            // backward meets its last use first
            const float2* tsl = trans + (size_t)stackIdx(sl) * sliceElems;
            float* dvs = dL_dV + (size_t)stackIdx(sl) * sliceElems;
            const bool acc = sl != lastUse[stackIdx(sl)];
            if (det)
                QS_TRY(launch_dv_gather(grad_t, npos, nx, ny, P.potNx, P.potNy, d_pos, d_pos + npos, tsl, sigma,
                                        d_part, dvs, acc, s));
            else
                QS_TRY(launch_dv_from_sum((float2*)d_part, P.potNx, P.potNy, tsl, sigma, dvs, acc, s));
        }
    }
    if (loss) {
        std::vector<double> h(nLoss);
        QS_CUDA_TRY(cudaMemcpyAsync(h.data(), d_loss, sizeof(double) * nLoss, cudaMemcpyDeviceToHost, s));
        QS_CUDA_TRY(cudaStreamSynchronize(s));
        double t = 0;
        for (double v : h) t += v;
        *loss = t;
    } else if (flags & QS_SYNC) {
        QS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return QS_OK;
}

int qs_atoms_grad(qs_ctx* c, const qs_params* p, const qs_atom* atoms, int natom, const float* dL_dV,
                  double* grad_xy, unsigned flags) {
    if (!c || !dL_dV || !grad_xy || (natom > 0 && !atoms)) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    if (!p->fftpotential || !p->potential3D) {
        set_error("only the 3-D FFT-integrated potential is supported");
        return QS_ERR_UNSUPPORTED;
    }
    QS_CUDA_TRY(cudaSetDevice(c->device));
    // a cell divided into slabs with one stack per slab: every slab's atom
    // placement against its own dL/dV, summed; otherwise slab 0's (the stack
    // the forward reused for every slab)
    const int nslab = (p->cellDiv > 1 && (flags & QS_SLAB_STACKS)) ? p->cellDiv : 1;
    const size_t stackElems = (size_t)p->slices * p->potNx * p->potNy;
    std::vector<double> total(2 * (size_t)std::max(natom, 1), 0.0), part(total.size());
    void* dg = nullptr;
    QS_TRY(ensure(c, B_OUT3, sizeof(double) * 2 * std::max(natom, 1), &dg));
    for (int slab = 0; slab < nslab; slab++) {
        std::vector<AtomJob> jobs;
        std::vector<std::pair<int, double>> lutKeys;
        plan_atoms(*p, atoms, natom, jobs, lutKeys, slab);
        QS_CUDA_TRY(cudaMemsetAsync(dg, 0, sizeof(double) * 2 * std::max(natom, 1), c->stream));
        if (!jobs.empty()) {
            int Nz = 0, Nr = 0, ns = 0;
            const float* const* d_luts = nullptr;
            QS_TRY(prepare_luts(c, *p, lutKeys, &d_luts, &Nz, &Nr, &ns));
            void* dj = nullptr;
            QS_TRY(ensure(c, B_JOBS, sizeof(AtomJob) * jobs.size(), &dj));
            QS_CUDA_TRY(cudaMemcpyAsync(dj, jobs.data(), sizeof(AtomJob) * jobs.size(), cudaMemcpyHostToDevice,
                                        c->stream));
            QS_TRY(launch_atoms_grad((const AtomJob*)dj, (int)jobs.size(), d_luts, Nz, Nr, ns, *p,
                                     dL_dV + (size_t)slab * stackElems, (double*)dg, c->stream));
        }
        QS_CUDA_TRY(cudaMemcpyAsync(part.data(), dg, sizeof(double) * 2 * natom, cudaMemcpyDeviceToHost, c->stream));
        QS_CUDA_TRY(cudaStreamSynchronize(c->stream));
        for (size_t i = 0; i < 2 * (size_t)natom; i++) total[i] += part[i];
    }
    std::copy(total.begin(), total.begin() + 2 * (size_t)natom, grad_xy);
    return QS_OK;
}

int qs_collect(qs_ctx* c, const qs_params* p, const float* wave_k, double* det_sums, float* diffpat,
               unsigned flags) {
    if (!c || !wave_k) { set_error("null argument"); return QS_ERR_ARG; }
    QS_TRY(check_params(p));
    QS_CUDA_TRY(cudaSetDevice(c->device));
    const qs_params& P = *p;
    cudaStream_t s = c->stream;
    const size_t N = (size_t)P.nx * P.ny;
    const bool host = (flags & QS_HOST_IO) != 0;
    PropTables tb = prop_tables(P);
    void* dtab = nullptr;
    QS_TRY(ensure(c, B_TABLES, sizeof(float) * (P.nx + P.ny), &dtab));
    QS_CUDA_TRY(cudaMemcpyAsync(dtab, tb.kx2.data(), sizeof(float) * P.nx, cudaMemcpyHostToDevice, s));
    QS_CUDA_TRY(cudaMemcpyAsync((float*)dtab + P.nx, tb.ky2.data(), sizeof(float) * P.ny, cudaMemcpyHostToDevice, s));
    const float2* w = (const float2*)wave_k;
    if (host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_DIFF_IN, sizeof(float2) * N, &d));
        QS_CUDA_TRY(cudaMemcpyAsync(d, wave_k, sizeof(float2) * N, cudaMemcpyHostToDevice, s));
        w = (const float2*)d;
    }
    void* dsum = nullptr;
    QS_TRY(ensure(c, B_SUM, sizeof(double) * QS_MAX_DETECTORS, &dsum));
    float* dp = diffpat;
    if (diffpat && host) {
        void* d = nullptr;
        QS_TRY(ensure(c, B_OUT2, sizeof(float) * N, &d));
        dp = (float*)d;
    }
    QS_TRY(launch_collect(P, w, (float*)dtab, (float*)dtab + P.nx, (double*)dsum, dp, s));
    if (det_sums && P.detectorNum > 0)
        QS_CUDA_TRY(cudaMemcpyAsync(det_sums, dsum, sizeof(double) * P.detectorNum,
                                    host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    if (diffpat && host) QS_CUDA_TRY(cudaMemcpyAsync(diffpat, dp, sizeof(float) * N, cudaMemcpyDeviceToHost, s));
    if (host || (flags & QS_SYNC)) QS_CUDA_TRY(cudaStreamSynchronize(s));
    return QS_OK;
}

}  // extern "C"
