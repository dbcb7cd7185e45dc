// qs_internal.h -- declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/qstem_gpu.h"

namespace qs {

// ------------------------------------------------------------- errors
void set_error(const std::string& msg);
// process-wide count of kernels this library launched (for measurement)
void count_launch(int n);
// Raise `func`'s dynamic shared-memory limit to `bytes` on the current
// device (once per device and kernel; a limit is a property of one context).
int smem_attr(const void* func, size_t bytes);
// CTAs of `func` resident per SM on the current device, and its SM count.
int resident_ctas(const void* func, int threads, size_t bytes, int* ctas, int* sms);
#define QS_CUDA_TRY(expr)                                                               \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            ::qs::set_error(std::string(#expr " failed: ") + cudaGetErrorString(_e));   \
            return QS_ERR_CUDA;                                                         \
        }                                                                               \
    } while (0)
#define QS_TRY(expr)              \
    do {                          \
        int _rc = (expr);         \
        if (_rc != QS_OK) return _rc; \
    } while (0)

// ------------------------------------------------- shared host-side checks
// The checks every entry point makes on qs_params (grid, sampling, energy,
// slabs, sequence, outputs, detectors).
int check_params(const qs_params* p);
// A batch without window offsets or without detector pixels takes them from
// the scan raster, which then needs scanXN, scanYN >= 1.
int check_raster(const qs_params& p, const qs_batch& b, bool wantDetPixels);
// wavelength (stem3/stemutil.cpp:714-725), Angstrom
double wavelength(double kev);

// propagate_slow's tables (stem3/stemlib.cpp:2783-2824) in the reference's
// float arithmetic
struct PropTables {
    std::vector<float> kx2, ky2;
    std::vector<float2> px, py;
    float k2max;
};
PropTables prop_tables(const qs_params& p);
// The ky columns the 2/3 band limit keeps: iy <= yA || iy >= yB (yA = yB = ny
// when the in-band set is not of that form, so that every column is kept),
// and the starts of the column tiles of width `colTile` that hold one.
struct Band {
    int yA, yB;
    std::vector<int> tiles;
};
Band band_tiles(const PropTables& t, int ny, int colTile);

// ------------------------------------------------------ multislice step
// Arguments of one row pass (transforms along y, the contiguous index).
enum RowMode { ROW_FIRST = 0, ROW_MID = 1, ROW_LAST = 2 };

// (RowCore is what the single-sampling row kernels take: the same kernel
// source given the larger RowArgs compiled to a 17 % slower 512^2 pass)
struct RowCore {
    int nx, ny, potNx, potNy;
    int nwaves;
    const float2* trans_slice;   // potNx x potNy c64 of the slice applied here
    size_t trans_stride;         // elements between the stacks of consecutive waves (0: one shared stack)
    const float2* probe;         // nx x ny (ROW_FIRST)
    size_t probe_stride;         // elements between consecutive waves' incident waves (0: shared)
    float2* waves;               // nwaves x nx x ny
    float2* waves_out;           // where ROW_FIRST/ROW_MID write (nullptr: in place)
    float2* exit_waves;          // ROW_LAST destination (may alias waves)
    const int* posX;             // nwaves window offsets
    const int* posY;
    const float2* tw;            // twiddle table of the length-ny line transform
    int yA, yB;                  // ky index in band iff iy <= yA || iy >= yB
    float norm;                  // 1/(nx*ny)
};
struct RowArgs : RowCore {
    // waves of different samplings in one launch (both set, or both null):
    const int2* band;            // per-wave (yA, yB) in place of yA, yB
    const int* step_slice;       // per-wave slice of its stack this step transmits
                                 // (trans_slice then points at slice 0)
};

// Arguments of one column pass (transforms along x).
struct ColArgs {
    int nx, ny, nwaves;
    float2* waves;
    float2* waves_out;           // where the inverse transform is stored (nullptr: in place)
    const float2* tw;            // twiddle table of the length-nx line transform
    const float* kx2;            // nx, float as propagate_slow computes
    const float* ky2;            // ny
    const float2* px;            // nx propagator factors (cos t, -sin t)
    const float2* py;            // ny
    float k2max;
    const int* tiles;            // column tile starts (ky0) of the in-band tiles
    int ntiles;
    int inverse;                 // 1: inverse x-transform and store; 0: k-space only
    // detectors (active when ndet > 0)
    int ndet;
    float k2in[QS_MAX_DETECTORS], k2out[QS_MAX_DETECTORS];
    double* partial;             // [nwaves][ntiles][ndet]
    float* diffpat;              // [nwaves][nx][ny] or null
    double scaleDiff;
    // waves of different samplings in one launch (no detectors):
    const int2* items;           // (wave, first column) of each work item, or null
    long nitems;                 // their number
    int per_wave;                // kx2, ky2, px, py hold one table per wave (nx or ny apart)
    const float* k2max_w;        // per-wave k2max, or null
};

// The whole slice loop of 256 x 256 waves in one launch, each wave held by a
// cluster of four CTAs in distributed shared memory (qs_resident.cu).
struct ResidentArgs {
    int potNx, potNy, nwaves, nsteps;
    const float2* trans;         // stack (slice a at a*potNx*potNy)
    size_t trans_stride;         // elements between the stacks of consecutive waves (0: shared)
    const float2* probe;         // incident waves, 256 x 256
    size_t probe_stride;         // elements between consecutive waves' incident waves (0: shared)
    const int* posX;             // nwaves window offsets
    const int* posY;
    const int* step_slice;       // nsteps: the stack slice each step transmits
    const int* step_slot;        // nsteps: the thickness slot a step writes, or -1
    const float2* tw;            // twiddles of the length-256 line transform
    int yA, yB, nb;              // band (as RowCore) and its number of columns
    const float* kx2;
    const float* ky2;
    const float2* px;
    const float2* py;
    float k2max;
    int ndet;
    float k2in[QS_MAX_DETECTORS], k2out[QS_MAX_DETECTORS];
    double* partial;             // [slot][nwaves][4][ndet], partial_slot elements per slot
    size_t partial_slot;
    float* diffpat;              // patterns: per slot (series, dp_slot apart) or of the last step
    size_t dp_slot;
    int series;
    float2* exit_waves;          // real-space waves after the last step, or null
    float norm;                  // 1/(nx*ny)
    double scaleDiff;
};
// clusters of the resident loop that fit on the current device at once
int resident_clusters(int* out);
// band columns the resident loop holds at most
int resident_band_columns();
int launch_resident(const ResidentArgs& a, cudaStream_t s);

int launch_rows(const RowArgs& a, RowMode mode, cudaStream_t s);
int launch_cols(const ColArgs& a, cudaStream_t s);
int col_tile_width(int nx);
int launch_det_finalize(const double* partial, int nwaves, int ntiles, int ndet, double scale,
                        const int* detPosX, const int* detPosY, int scanYN, int npix, float* det_out,
                        cudaStream_t s);

// in-place line transforms of `nlines` contiguous lines of length n
int line_fft_rows(float2* data, int n, long nlines, bool inverse, cudaStream_t s);
// generic in-place 2-D transform of `howmany` n0 x n1 arrays
int fft2d(float2* data, int n0, int n1, int howmany, bool inverse, cudaStream_t s);
int bandlimit_lines(float2* data, int n0, int n1, int howmany, const float* kx2, const float* ky2,
                    const float2* px, const float2* py, const int* tiles, int ntiles, int yA, int yB, float k2max,
                    cudaStream_t s);
// the row passes of bandlimit_lines (qs_rows.cu): forward with only the
// in-band columns stored (inverse false), or inverse from the in-band columns
int bandlimit_rows(float2* data, int n, long nlines, int yA, int yB, bool inverse, cudaStream_t s);
// in-place 2-D DFT of any size as batched complex matrix products (for
// potential grids the line FFTs do not cover); scratch holds scratch_slices
// n0 x n1 arrays
int dft2d(float2* data, int n0, int n1, int howmany, bool inverse, float2* scratch, int scratch_slices,
          cudaStream_t s);
// inter-pass twiddle table of the length-n row (col = false) or column
// (col = true) line transform (per-pass layout of LineCfg), device-resident
// and cached per device, n and kind; twiddle_host fills the same table on the
// host
const float2* twiddles(int n, bool col = false);
int twiddle_host(int n, std::vector<float2>& h, bool col = false);

// ---------------------------------------------------------- potentials
struct LutTable {
    float* d_lut = nullptr;  // Nz x Nr
    int Nz = 0, Nr = 0, nzSub = 0;
};
int build_lut(const qs_params& p, int Z, double B, int charged, float* d_out, int* Nz, int* Nr,
              int* nzSub, cudaStream_t s);

struct AtomJob {
    int index;                   // the atom's position in the caller's array
    float atomX, atomY, atomZ;   // atomZ after the reference's offsets
    float q;
    int iax0, iax1, iay0, iay1;  // inclusive pixel box (unwrapped coordinates)
    int iaz0, iaz1;              // slice range relative to iAtomZ
    int iAtomZ;
    int lut, lutq;               // LUT indices (-1: none)
};
// One atom of the periodic 2-D potential (make3DSlices' 2-D branch): its
// slice, the unwrapped first pixel of its 2 iRadX x 2 iRadY box, the table
// offsets and the bilinear weights, as the reference forms them.
struct Atom2DJob {
    double s11, s12, s21, s22;
    int lut, iAtomZ, iax0, iay0, iOffsX, iOffsY;
};
// getAtomPotential2D: nx x ny real parts (float) into d_out (null: sizes only)
int build_lut2d(const qs_params& p, int Z, double B, float* d_out, int* nx, int* ny, cudaStream_t s);
int launch_scatter2d(const Atom2DJob* d_jobs, int njobs, const float* const* d_luts, int nyAtBox, int boxX, int boxY,
                     const qs_params& p, float* V, cudaStream_t s);
// the scatter-sum into V[slices][potNx][potNy] (float, zeroed by the caller);
// charged: some job has a charge LUT (lutq >= 0)
int launch_scatter(const AtomJob* d_jobs, int njobs, bool charged, const float* const* d_luts, int Nz, int Nr,
                   int nzSub, const qs_params& p, const double* d_knots, float* V, cudaStream_t s);
// Akima's local cubic spline coefficients of (x, y), n >= 4 knots
// (stem3/stemutil.cpp:975-1041)
void akima_spline(const double* x, const double* y, double* b, double* c, double* d, int n);
// make3DSlicesFT's potential (custom scattering factors k[nk], f[kind][nk]
// of the elements Zs[kind]) into the real array V[slices][potNx][potNy]
// (qs_custom.cu); synchronises the stream
int build_custom_potential(const qs_params& P, const qs_atom* atoms, int natom, const double* k, int nk,
                           const int* Zs, const double* sf, int nkinds, float* V, cudaStream_t s);
// knots[k], k = 0..Nr: the smallest s = x^2 + y^2 (double) whose radial
// interval floor(fl(fl(sqrt(s)) / dr)) in make3DSlices is at least k
void scatter_knots(double dr, int Nr, std::vector<double>& knots);
// trans = (V, 0)
int launch_expand_real(const float* V, float2* trans, size_t n, cudaStream_t s);
int launch_bandlimit_mask(float2* trans, int slices, int potNx, int potNy, const float* kx2,
                          const float* ky2, float k2max, double fftScale, cudaStream_t s);

// ---------------------------------------------------------------- probe
int launch_probe_kspace(const qs_params& p, double dx, double dy, float2* wave, cudaStream_t s);
int launch_probe_realspace(const qs_params& p, double dx, double dy, float2* wave, double* d_sum,
                           cudaStream_t s);
int launch_scale_by_sum(float2* wave, size_t n, const double* d_sum, double nxy, cudaStream_t s);

// ----------------------------------------------------------------- adjoint
struct AdjLastArgs {
    int nx, ny, nwaves, yA, yB;
    const float2* waves;         // state after the last row pass
    float2* waves_out;           // g_A of the last slice
    const float2* tw;            // twiddles of the length-nx transform
    const float *kx2, *ky2;
    const float2 *px, *py;       // forward propagator factors
    float k2max;
    const float* target;         // [nwaves][nx][ny], fftshifted like diffpat
    float* diffpat;              // optional forward patterns
    double scaleDiff;            // 1/sqrt(nx*ny)
    double* loss_partial;        // [nwaves * ny/C]
};
struct AdjRowArgs {
    int nx, ny, potNx, potNy, nwaves, yA, yB;
    float2* grad;                // in: g_A, out: g_h (band-limited columns)
    const float2* state;         // h of this slice (not read for the first slice)
    const float2* probe;         // first slice
    const float2* trans_slice;
    float2* grad_t;              // out: conj(psi) g_phi, [nwaves][nx][ny] (gsum == nullptr)
    float2* gsum;                // or: conj(psi) g_phi added into its window of this
                                 // potNx x potNy sum (float atomics, any order)
    const int *posX, *posY;
    const float2* tw;            // twiddles of the length-ny transform
    float norm;
};
int launch_adj_last(const AdjLastArgs& a, cudaStream_t s);
int launch_adj_rows(const AdjRowArgs& a, bool first, cudaStream_t s);
// dL/dV of one slice from the per-position g_t: positions are summed in
// chunks into `partial` (dv_partial_bytes), then reduced
size_t dv_partial_bytes(int npos, int potNx, int potNy);
int launch_dv_gather(const float2* grad_t, int npos, int nx, int ny, int potNx, int potNy, const int* posX,
                     const int* posY, const float2* trans_slice, double sigma, void* partial, float* dV,
                     bool accumulate,
                     cudaStream_t s);
// dL/dV of one slice from the summed windows G (gsum of the row adjoint):
// dV (=|+=) -2 sigma Im(conj(G) t), and G cleared for the next slice
int launch_dv_from_sum(float2* gsum, int potNx, int potNy, const float2* trans_slice, double sigma, float* dV,
                       bool accumulate, cudaStream_t s);
int launch_atoms_grad(const AtomJob* d_jobs, int njobs, const float* const* d_luts, int Nz, int Nr, int nzSub,
                      const qs_params& p, const float* dV, double* grad, cudaStream_t s);
int launch_grating_from_real(const float* V, float2* trans, size_t n, double scale, cudaStream_t s);

// ------------------------------------------------------------------- TEM
int launch_fill(float2* w, size_t n, float re, float im, cudaStream_t s);
// acc[i] += scale * sum over nwaves arrays (n apart) of |w[i]|^2
int launch_acc_intensity(const float2* w, int nwaves, size_t n, float scale, float* acc, cudaStream_t s);
// out_b = in_b * H elementwise, b < nwaves
int launch_mul_table(const float2* in, const float2* H, int nwaves, size_t n, float2* out, cudaStream_t s);
// objective-lens transfer H(k) of defocus df on an nx x ny grid (FFT order)
int launch_ctf_table(int nx, int ny, double dx, double dy, double lambda, const qs_ctf& C, double df, float2* H,
                     cudaStream_t s);

// collectIntensity for one k-space wave (compat entry point)
int launch_collect(const qs_params& p, const float2* wave_k, const float* kx2, const float* ky2,
                   double* d_sums, float* diffpat, cudaStream_t s);

}  // namespace qs
