/*
 * qstem_gpu.h -- C ABI of the GB300 multislice library (libqstem_gpu.so).
 *
 * This is the drop-in boundary for QSTEM's multislice hot path in
 * stem3/stemlib.cpp.  Each entry point replaces one reference function of the
 * call surface declared in stem3/stemlib.h:
 *
 *   qs_lut_build        getAtomPotential3D / getAtomPotentialOffset3D
 *                       (stem3/stemlib.h:51-52; stem3/stemlib.cpp:1342, :1548)
 *   qs_slices_build     make3DSlices + initSTEMSlices (qs_slab_build: one slab
 *                       of a cell divided along z)
 *                       (stem3/stemlib.h:45, :39; stem3/stemlib.cpp:383, :2199)
 *   qs_slices_build_custom  make3DSlicesFT + initSTEMSlices: custom
 *                       scattering factors (stem3/customslice.h:28;
 *                       stem3/customslice.cpp:56)
 *   qs_probe            probe (stem3/stemlib.h:36; stem3/stemlib.cpp:1952)
 *   qs_multislice_run   the position loop of doSTEM/doCBED around runMulsSTEM,
 *                       which fuses transmit, the 2-D FFT pair, propagate_slow,
 *                       fft_normalize and collectIntensity
 *                       (stem3/stem3.cpp:2820-2946; stem3/stemlib.h:64, :41,
 *                        :48-49, :66; stem3/stemlib.cpp:2375, :2576, :2760,
 *                        :2867, :2890)
 *   qs_collect          collectIntensity for one k-space wave
 *                       (stem3/stemlib.h:41; stem3/stemlib.cpp:2576)
 *   qs_cbed_batch_run   doCBED (stem3/stem3.cpp:2048-2344) for many independent
 *                       instances of mixed grids, thicknesses and optics in
 *                       one call, admitted by device-memory footprint
 *   qs_tem_run          doTEM's configuration loop (stem3/stem3.cpp:2354-2710):
 *                       plane wave, every frozen-phonon configuration as one
 *                       batch, exit-wave intensity average, and the
 *                       through-focus CTF images of
 *                       GUI_Matlab/simImageFromWave.m:57-73
 *
 * Conventions
 *   - Plain C types only; complex numbers are interleaved float pairs
 *     [re, im] ("c64"), matching fftwf_complex.
 *   - Arrays are row-major [x][y] with y fastest, as the reference's
 *     complex2Df/complex3Df allocators lay them out
 *     (libs/memory_fftw3.cpp:446, :523): wave[ix][iy], trans[z][ix][iy].
 *   - Every function returns an int status: QS_OK (0) or a negative
 *     QS_ERR_* code; qs_last_error() returns the message of the calling
 *     thread's last failure.  Nothing calls exit(): the reference's
 *     printf+exit(0) error paths become error codes.
 *   - All buffers are owned by the caller.  Pointer arguments are device
 *     pointers unless the `flags` argument carries QS_HOST_IO, in which case
 *     they are host pointers and the library copies through its own device
 *     staging buffers.
 *   - A context owns one CUDA stream on one device; calls on one context are
 *     serialised on that stream, different contexts may be used from
 *     different threads.
 */
#ifndef QSTEM_GPU_H
#define QSTEM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QS_ABI_VERSION 3

/* status codes */
#define QS_OK 0
#define QS_ERR_ARG (-1)         /* invalid argument or inconsistent parameters */
#define QS_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define QS_ERR_NOMEM (-3)       /* device allocation refused (admission control) */
#define QS_ERR_UNSUPPORTED (-4) /* a size or option this build does not implement */
#define QS_ERR_TIMEOUT (-5)     /* a bounded device wait gave up */

/* flags */
#define QS_HOST_IO 1u           /* buffer pointers are host memory */
#define QS_OUT_POTENTIAL 2u     /* qs_slices_build: stop after make3DSlices (V in .re) */
#define QS_SYNC 4u              /* synchronise the stream before returning */
#define QS_SLAB_STACKS 8u       /* qs_multislice_run with cellDiv > 1: trans holds one
                                   slices-long stack per slab, back to back */
#define QS_SERIES 16u           /* qs_multislice_run: diffpats and exit_waves hold one
                                   array per thickness slot, [tCount+1][npos][nx][ny] */
#define QS_GRAPH 32u            /* qs_multislice_run with device buffers: replay the slice
                                   loop as a CUDA graph (captured on the second call with
                                   the same parameters, buffers and batch) */
#define QS_DETERMINISTIC 64u    /* qs_adjoint_run: sum dL/dV over positions in a fixed order
                                   (bit-reproducible, slower) instead of with float atomics */
#define QS_RESIDENT 128u        /* qs_multislice_run with 256 x 256 waves: the whole slice
                                   loop in one launch, each wave held on chip by a cluster
                                   of four CTAs for all of its slices, instead of a row and
                                   a column pass per slice through HBM (measured slower:
                                   the passes are issue-bound, not HBM-bound, at 256^2) */

/* run modes, same numbering as libs/stemtypes_fftw3.h:35-42 */
#define QS_MODE_STEM 1
#define QS_MODE_CBED 2
#define QS_MODE_TEM 3

#define QS_MAX_DETECTORS 16

/* One atom; identical layout to the reference's `atom`
 * (libs/stemtypes_fftw3.h:70-77), z first. 28 bytes. */
typedef struct qs_atom {
    float z, y, x;
    float dw;   /* Debye-Waller factor B (A^2) */
    float occ;  /* occupancy */
    float q;    /* charge */
    int Znum;   /* atomic number, 0 = vacancy */
} qs_atom;

/* One annular detector; the fields the reference's Detector carries for
 * collectIntensity (libs/data_containers.h:77-97).  k2Inside/k2Outside are
 * (sin(r*1e-3)/lambda)^2 rounded to float as stem3/stem3.cpp:1343-1350 does;
 * qs_params_finalize fills them from rInside/rOutside. */
typedef struct qs_detector {
    float rInside, rOutside; /* mrad */
    float k2Inside, k2Outside;
    float shiftX, shiftY;    /* pixels */
} qs_detector;

/* The MULS fields the hot path reads (libs/data_containers.h:103-308), with
 * the reference's own types (float where MULS has float_tt) so that the
 * arithmetic can reproduce it. */
typedef struct qs_params {
    int mode;               /* QS_MODE_* */
    int nx, ny;             /* wave grid */
    int potNx, potNy;       /* potential/transmission grid */
    int slices;             /* slices per stack */
    int cellDiv;            /* slabs the cell is divided into along z (NCELLZ: n/cellDiv) */
    int outputInterval;     /* "slices between outputs" */
    int centerSlices, nonPeriod, nonPeriodZ, potential3D, fftpotential;
    int bandlimittrans, tds;
    float resolutionX, resolutionY; /* A/pixel */
    float sliceThickness;   /* A */
    float czOffset;         /* zOffset: A */
    float potOffsetX, potOffsetY;
    float potSizeX, potSizeY;
    float ax, by, c;        /* super-cell size, A */
    float atomRadius;       /* A */
    float v0;               /* kV */
    /* probe optics (stem3/stem3.cpp:1120-1275); lengths in A, angles rad */
    float alpha;            /* mrad */
    float Cs, C5, df0, astigMag, astigAngle, Cc, dE_E;
    float a33, a31, a44, a42, a55, a53, a51, a66, a64, a62;
    float phi33, phi31, phi44, phi42, phi55, phi53, phi51, phi66, phi64, phi62;
    int ismoth, gaussFlag;
    float gaussScale;
    float aAIS;
    /* scan (stem3/stem3.cpp:1054-1068, adjusted as :1436-1446) */
    float scanXStart, scanXStop, scanYStart, scanYStop;
    int scanXN, scanYN;
    float electronScale;    /* beam current * dwell time * MILLISEC_PICOAMP */
    int detectorNum;
    qs_detector detectors[QS_MAX_DETECTORS];
    /* readFile's equalDivs (stem3/stem3.cpp:930-931): with cellDiv > 1, every
     * slab has the potential of slab 0, built once and reused */
    int equalDivs;
    /* The stacking sequence "sequence: m1 m2" (stem3/stem3.cpp:2761-2790,
     * stem3/stemlib.cpp:2403-2429): the wave passes m2 times through the
     * cellDiv slabs, and through each slab's stack m1 times in a row.  The
     * thickness slot of a step is collectIntensity's t of the index
     * totalSliceCount + islice*(1 + repeat) the reference passes it.
     * qs_multislice_run, qs_stem_run, qs_tem_run, qs_cbed_batch_run and
     * qs_adjoint_run (a stack slice's dL/dV sums all its steps) walk the
     * sequence; the no-allocation entry point takes "1 1" only (QS_ERR_ARG).
     * 0 reads as 1. */
    int mulsRepeat1, mulsRepeat2;
} qs_params;

/* A batch of probe positions for qs_multislice_run.  Position p uses the
 * transmission window at integer offset (iPosX[p], iPosY[p]) of the
 * potNx x potNy stack and writes detector pixel (detPosX[p], detPosY[p])
 * (the WAVEFUNC fields of the same names, libs/data_containers.h:35-37).
 * All four arrays are HOST arrays of length npos.  A NULL iPosX/iPosY
 * computes the offsets of a full scan_x/scan_y raster the way doSTEM does
 * (stem3/stem3.cpp:2860-2871) with p = ix*scanYN + iy. */
typedef struct qs_batch {
    int npos;
    const int *iPosX, *iPosY;
    const int *detPosX, *detPosY;
} qs_batch;

typedef struct qs_ctx qs_ctx;

/* ---------------------------------------------------------------- context */
int qs_ctx_create(int device, qs_ctx **out);
int qs_ctx_destroy(qs_ctx *ctx);
const char *qs_last_error(void);
int qs_abi_version(void);
/* The stream the context launches on (a cudaStream_t, as an opaque pointer). */
void *qs_ctx_stream(qs_ctx *ctx);
/* Fill derived fields (detector k2 bounds) exactly as readFile does. */
int qs_params_finalize(qs_params *p);
/* Number of thickness outputs tCount+1 (stem3/stemlib.cpp:2589). */
int qs_thickness_count(const qs_params *p);

/* ------------------------------------------------------------ potentials */
/* Projected-potential lookup table of one element: Nz_lut x Nr floats
 * (the real parts of the reference's complex LUT).  `charged` selects the
 * charge-derivative table of getAtomPotentialOffset3D.  B is the
 * Debye-Waller factor.  out may be NULL to query the dimensions. */
int qs_lut_build(qs_ctx *ctx, const qs_params *p, int Znum, double B, int charged,
                 float *out, int *Nz_lut, int *Nr, int *nzSub, unsigned flags);

/* Build trans[slices][potNx][potNy] (c64) from `natom` atoms: the
 * scatter-sum of make3DSlices followed by initSTEMSlices' exp(i*lambda*gamma*V)
 * and optional band limit.  With QS_OUT_POTENTIAL the result stops after the
 * scatter-sum (V in .re, 0 in .im).  atoms is a host array. */
int qs_slices_build(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, int natom,
                    float *trans, unsigned flags);

/* The same for slab `slab` (0 <= slab < cellDiv) of a cell divided into
 * cellDiv slabs along z: make3DSlices' successive calls, which offset the
 * atoms by -slab * slices * sliceThickness (stem3/stemlib.cpp:456-465,
 * :709-713).  qs_slices_build is slab 0. */
int qs_slab_build(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, int natom, int slab,
                  float *trans, unsigned flags);

/* The same from custom scattering factors ("Structure Factors: custom"):
 * make3DSlicesFT (stem3/customslice.cpp:56-317), the path doCBED and doNBED
 * take for them (stem3/stem3.cpp:2177-2197), followed by initSTEMSlices.
 * k[nk] (1/A) and f[kind][nk] (A) are the table readSFactLUT reads
 * (stem3/stem3.cpp:555-600: "Nk:", "k:", one line per element), for the
 * elements Z[kind]; every atom's element must be among them.  The potential
 * of each element is the inverse 2-D FFT of f on a 40 A (z, r) box, cut off
 * where it first turns negative, interpolated bicubically for every atom,
 * pixel and slice within the cut-off (a brute force, as in the reference).
 * potential3D and cellDiv do not change it (the reference builds slab 0's
 * stack on every call); slices must be at least 2 (the reference adds no
 * atom to a single slice).  Flags as for qs_slices_build. */
int qs_slices_build_custom(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, int natom, const double *k,
                           int nk, const int *Z, const double *f, int nkinds, float *trans, unsigned flags);

/* ----------------------------------------------------------------- probe */
/* nx x ny c64 real-space probe centred at (dx, dy) A. */
int qs_probe(qs_ctx *ctx, const qs_params *p, double dx, double dy, float *wave,
             unsigned flags);

/* ------------------------------------------------------------ multislice */
/* Run every position of `batch` through all slices of `trans` (device,
 * slices x potNx x potNy c64), starting from `probe` (device nx x ny c64,
 * NULL = build the centred probe).  With cellDiv > 1 the wave continues
 * through cellDiv slabs (doSTEM's slab loop, stem3/stem3.cpp:2795-2949), the
 * thickness slots counting absolute slices: `trans` is one stack reused for
 * every slab, or with QS_SLAB_STACKS cellDiv stacks back to back
 * (qs_slab_build).  Outputs (each may be NULL):
 *   det_images  [tCount+1][detectorNum][scanXN][scanYN] float, the
 *               detector images after the last slice of each thickness
 *               group (collectIntensity's overwrite semantics)
 *   diffpats    [npos][nx][ny] float, fftshifted |psi(k)|^2/sqrt(nx*ny) of
 *               the final slice (wave->diffpat)
 *   exit_waves  [npos][nx][ny] c64 real-space exit waves
 * With QS_SERIES diffpats and exit_waves get a leading thickness-slot axis
 * ([tCount+1][npos][nx][ny]): slot t holds the pattern / real-space wave
 * after the slice that writes detector slot t, i.e. collectIntensity's
 * diff_<t>.img of CBED runs (stem3/stemlib.cpp:2663-2676) and, for the slots
 * interimWave writes, its wave_<t>.img (stem3/stemlib.cpp:2538-2565); the
 * last slot is the final slice's.
 * Each slice is a row pass and a column pass over the batch; with
 * QS_RESIDENT, 256 x 256 waves (without QS_SERIES exit waves) run the whole
 * loop in one launch with each wave resident on chip.
 * Buffers are device pointers, or host pointers with QS_HOST_IO. */
int qs_multislice_run(qs_ctx *ctx, const qs_params *p, const float *trans, const float *probe,
                      const qs_batch *batch, float *det_images, float *diffpats,
                      float *exit_waves, unsigned flags);

/* One frozen-phonon configuration of doSTEM end to end
 * (stem3/stem3.cpp:2795-2948): make3DSlices + initSTEMSlices from host
 * atoms into a context-owned device stack, then every position of `batch`
 * through qs_multislice_run.  Outputs are HOST buffers (as for QS_HOST_IO);
 * the transmission stack stays on the device.  The slice loop runs on the
 * context's own buffers with QS_GRAPH, so repeated configurations of the same
 * scan replay it as one CUDA graph. */
int qs_stem_run(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, int natom,
                const qs_batch *batch, float *det_images, float *diffpats);

/* ----------------------------------------------------------------- CBED */
/* One doCBED instance (stem3/stem3.cpp:2048-2344): mode CBED parameters
 * (potential grid = wave grid, qs_params as readFile fills them), the probe
 * at (scanXStart - potOffsetX, scanYStart - potOffsetY) (:2096-2100), host
 * atoms, and the HOST output: the fftshifted |psi(k)|^2/sqrt(nx*ny) after the
 * last slice (the collectIntensity pattern doCBED writes as diffAvg_1.img at
 * save level <= 1). */
typedef struct qs_cbed_job {
    qs_params params;
    const qs_atom *atoms;
    int natom;
    float *diffpat;          /* [nx][ny] */
} qs_cbed_job;

/* What the scheduler did. */
typedef struct qs_cbed_report {
    int groups;              /* batches of instances sharing a grid */
    int rounds;              /* admission rounds */
    int streams;             /* CUDA streams the groups of a round ran on */
    double admitted_bytes;   /* largest device footprint of a round */
    double budget_bytes;     /* the admission budget used */
} qs_cbed_report;

/* Run `njobs` independent CBED instances.  Instances with the same grid run
 * as one batch, one launch per pass and step for all of them: each wave has
 * its own slice stack, probe, propagator and k^2 tables (its sampling, slice
 * thickness and energy), band, thickness and stacking, and stops after its
 * own number of steps; the batches of a round run concurrently on separate
 * streams.  A round admits whole batches, largest first, while the sum of
 * their footprints (slice stacks + waves + probes + patterns + tables) fits
 * the budget: the free device memory less 1 GiB, or max_bytes if that is
 * smaller and not 0.  An instance that alone does not fit is rejected
 * (QS_ERR_NOMEM).  A cell divided into slabs (cellDiv > 1) runs through all
 * of them and a stacking sequence through its passes, as doCBED's slab loop
 * does: one stack is kept per slab (slab 0's alone for equal divisions) and
 * the steps index it.  report may be NULL. */
int qs_cbed_batch_run(qs_ctx *ctx, const qs_cbed_job *jobs, int njobs, size_t max_bytes,
                      qs_cbed_report *report);

/* ------------------------------------------------------------------ TEM */
/* Objective-lens transfer of GUI_Matlab/simImageFromWave.m:57-73 (lengths in
 * Angstrom, angles in radians, spatial frequencies in 1/Angstrom):
 *   H(k) = A(k) exp(-i pi (lambda (df + astig cos 2(phi - astigPhi)) k^2
 *                          + lambda^3 Cs k^4 / 2))
 *          exp(-2 (focalSpread lambda k^2)^2)                 temporal envelope
 *          exp(-(pi alpha df + pi alpha lambda^2 Cs k^2)^2 k^2) spatial envelope
 * A(k) = 1 for k < kmax - edge/2, 0 for k > kmax + edge/2, and a raised
 * cosine between (edge = 0: the script's hard aperture k^2 < kmax^2;
 * kmax <= 0: no aperture).  df is the defocus of each image. */
typedef struct qs_ctf {
    double Cs;           /* spherical aberration */
    double astig;        /* two-fold astigmatism magnitude */
    double astigPhi;     /* its azimuth */
    double focalSpread;  /* Cc * dE/E */
    double alpha;        /* illumination semi-angle */
    double kmax;         /* objective aperture radius */
    double edge;         /* width of the aperture's cosine edge */
} qs_ctf;

/* doTEM for `nconf` frozen-phonon configurations (stem3/stem3.cpp:2354-2710).
 * atoms holds the configurations back to back, natoms[c] atoms each (host).
 * Every configuration gets its own slice stack (make3DSlices +
 * initSTEMSlices; one per slab of a cell divided into unequal slabs), and
 * all of them run as one batch from doTEM's untilted incident plane wave
 * psi = 1 (:2403-2406) to their exit waves.
 * Outputs (HOST buffers, each may be NULL):
 *   mean_intensity  [nx][ny] float, the mean over configurations of
 *                   |psi_exit|^2 (doTEM's image.img holds (nx*ny)^2 times
 *                   its running mean: an unnormalised FFT round trip,
 *                   :2583-2608)
 *   ctf_images      [ndef][nx][ny] float, the mean over configurations of
 *                   |IFFT(FFT(psi_exit) H_df)|^2 for df = defoci[i]
 *   exit_waves      [nconf][nx][ny] c64 (doTEM's wave.img per configuration)
 * Configurations are batched as device memory allows. */
int qs_tem_run(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, const int *natoms, int nconf,
               const qs_ctf *ctf, int ndef, const double *defoci, float *mean_intensity,
               float *ctf_images, float *exit_waves);

/* qs_tem_run with doTEM's tilted incident plane wave (beam tilt btiltx,
 * btilty in rad, held as floats as MULS holds them;
 * stem3/stem3.cpp:2409-2419): psi(ix, iy) = exp(i k_t.(x, y)) with
 * k_t = 2 pi sin(tilt) / lambda, x = dx (ix - nx/2) and -- as the reference
 * forms it -- y = dy (ix - nx/2).  Exit waves are returned as propagated;
 * doTEM's tilt-back applies to the wave.img file only. */
int qs_tem_run_tilted(qs_ctx *ctx, const qs_params *p, double btiltx, double btilty, const qs_atom *atoms,
                      const int *natoms, int nconf, const qs_ctf *ctf, int ndef, const double *defoci,
                      float *mean_intensity, float *ctf_images, float *exit_waves);

/* ------------------------------------------------------------ gradients */
/* initSTEMSlices' phase grating for a given potential stack V
 * (stem3/stemlib.cpp:2280-2299): trans = exp(i*lambda*gamma*V), V a device
 * slices x potNx x potNy float array, trans a device c64 array (no band limit). */
int qs_phase_grating(qs_ctx *ctx, const qs_params *p, const float *V, float *trans, unsigned flags);

/* Differentiable 4D-STEM.  The reference has no adjoint; the forward model is
 * its runMulsSTEM (stem3/stemlib.cpp:2375-2534) for the positions of `batch`.
 * Loss L = sum_p sum_k (I_p(k) - target_p(k))^2, I_p the diffraction pattern
 * after the last slice (fftshifted |psi(k)|^2/sqrt(nx*ny), the layout of
 * qs_multislice_run's diffpats).  Writes L (host double, may be NULL),
 * dL/dV for every slice of the potential (device float,
 * slices x potNx x potNy, through t = exp(i*lambda*gamma*V)) and optionally
 * the forward patterns (device, [npos][nx][ny]).  Forward waves are kept every
 * `ckpt` slices and recomputed in between (1 = keep all; <= 0 = keep all when
 * they fit in free device memory less 1 GiB, else the smallest interval that
 * fits).  All arrays are device pointers; trans must not be band-limited.
 * A cell divided into slabs (cellDiv > 1) runs through all of them: trans is
 * one stack reused for every slab, whose dL/dV slices then sum the gradient
 * of every use, or with QS_SLAB_STACKS cellDiv stacks back to back and as
 * many dL/dV stacks.  The sum of dL/dV over positions uses float atomics
 * (the last bits depend on the order the GPU adds in); QS_DETERMINISTIC sums
 * in a fixed order instead. */
int qs_adjoint_run(qs_ctx *ctx, const qs_params *p, const float *trans, const float *probe,
                   const qs_batch *batch, const float *target, int ckpt, double *loss, float *dL_dV,
                   float *diffpats, unsigned flags);

/* dL/dx and dL/dy of every atom (grad_xy: host, natom x 2 doubles) from
 * dL/dV (device): the adjoint of make3DSlices' scatter-sum
 * (stem3/stemlib.cpp:894-1213) through its radial linear interpolation.
 * Atoms that contribute to no slice get zero; z gradients are not returned
 * (the LUT is nearest-neighbour in z, stem3/stemlib.cpp:76).  With
 * cellDiv > 1 and QS_SLAB_STACKS, dL_dV holds one stack per slab and the
 * gradients sum every slab's placement of the atoms (make3DSlices' offset
 * of slab k); without it, slab 0's (the stack reused for every slab). */
int qs_atoms_grad(qs_ctx *ctx, const qs_params *p, const qs_atom *atoms, int natom, const float *dL_dV,
                  double *grad_xy, unsigned flags);

/* ------------------------------------------------------------ profiling */
/* Per-context counters for measurement: kernel launches of this library and,
 * while profiling is enabled, CUDA-event times of the row and column passes
 * of the slice loop (recorded on the context's stream around each launch). */
typedef struct qs_stats {
    long long launches;        /* kernels launched by this context */
    long long row_launches, col_launches;
    double row_ms, col_ms;     /* summed event time of the passes */
    double row_bytes, col_bytes; /* algorithmic bytes of those passes */
} qs_stats;
int qs_ctx_profile(qs_ctx *ctx, int enable); /* resets the counters */
int qs_ctx_stats(qs_ctx *ctx, qs_stats *out); /* synchronises the stream */

/* ------------------------------------------------- without allocation */
/* No counterpart in the reference.  qs_multislice_run for callers that must
 * not allocate device memory while they run: cudaFree waits for the whole
 * device (stalling every other stream in the process), a framework's caching
 * allocator may own all device memory, or a deployment may have reserved its
 * whole budget up front.  This variant allocates nothing: besides the
 * caller's buffers it uses only a fixed scratch area of
 * QS_NOALLOC_SCRATCH_BYTES compiled into the library (held on every GPU that
 * loads the library until the process exits).
 *   - stream is a cudaStream_t (NULL: the default stream); all pointers are
 *     device pointers; probe is required (make it with qs_probe first).
 *   - Limit: the scratch holds the whole batch -- about nx*ny*8 bytes per
 *     position plus small tables -- so a 512x512 batch takes at most ~30
 *     positions, 256x256 ~120; larger batches are rejected with QS_ERR_ARG and
 *     a message giving the bytes needed.  Split the scan into such batches.
 *   - The first call on each device looks up the scratch address with
 *     cudaGetSymbolAddress; make that first call before any stream capture.
 *     Later calls can be captured into a CUDA graph: they copy nothing from
 *     host memory (tables and positions travel as kernel arguments), so a
 *     replay reads the buffers' current contents.
 *   - All calls share the one scratch area, which keeps the previous call's
 *     contents (the call clears what must start at zero): calls whose GPU work
 *     overlaps race on it and must be serialised by the caller. */
#define QS_NOALLOC_SCRATCH_BYTES (64u * 1024u * 1024u)
int qs_multislice_run_noalloc(void *stream, const qs_params *p, const float *trans, const float *probe,
                              const qs_batch *batch, float *det_images, float *diffpats,
                              float *exit_waves);

/* collectIntensity for one wave already in k-space (after propagate):
 * det_sums[d] = sum of |psi(k)|^2 over detector d's annulus (double, not yet
 * multiplied by electronScale/(nx*ny)^2, the factor the reference applies,
 * stem3/stemlib.cpp:2587), shifted detectors included; diffpat (may be NULL)
 * receives the fftshifted |psi(k)|^2/sqrt(nx*ny). */
int qs_collect(qs_ctx *ctx, const qs_params *p, const float *wave_k, double *det_sums,
               float *diffpat, unsigned flags);

#ifdef __cplusplus
}
#endif
#endif
