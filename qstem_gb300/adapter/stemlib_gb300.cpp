// stemlib_gb300.cpp -- drop-in for the multislice hot path of QSTEM's stem3.
//
// Compiled into the reference's stem3 program in place of the bodies of five
// functions of stem3/stemlib.cpp (declared in stem3/stemlib.h:36-64):
//
//   make3DSlices      atom handling as the reference does it (re-read and
//                     displaced per run, centring, z sort, the .cfg file),
//                     then qs_slices_build on the GPU (scatter-sum, phase
//                     grating and band limit; the stack stays on the device)
//   initSTEMSlices    nothing left to do (fused into qs_slices_build)
//   probe             qs_probe into wave->wave
//   runMulsSTEM       one position through qs_multislice_run on the calling
//                     thread's own context: exit wave, diffraction pattern,
//                     the position's detector pixels in every thickness slot,
//                     intIntensity, and the reference's wave file when it
//                     would write one
//   collectIntensity  qs_collect for one k-space wave
//
// stem3.cpp links unchanged: the reference's own five bodies are compiled
// under other names (oracle/Makefile, target `adapter`).  doSTEM's OpenMP
// position loop calls runMulsSTEM from several threads at once, so every
// thread gets its own context (one CUDA stream) and device buffers; the slice
// stack is shared read-only.
//
// Slabs (cellDiv > 1) run as the reference runs them: doSTEM builds each
// slab's stack before its pass (make3DSlices offsets the atoms by the slab's
// height) and hands every pass the previous pass's exit wave, so each call
// of runMulsSTEM transmits one slab.  It runs that slab with a thickness slot
// after every slice and files each slice's detector values under the slot
// collectIntensity would use, from the index muls->totalSliceCount + slice
// (stem3/stemlib.cpp:2591-2610), the last slice of a slot winning.  The
// sequence's inner repeat (mulsRepeat1 > 1) is not taken here (the library's
// one-call entry points walk it); the reference's optional potential dumps
// (savePotential) and the real-space interim files of save level > 1 in TEM
// and CBED mode are not written.  Errors print the library's message and
// exit, as the reference's own error paths do.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <vector>

#include <cuda_runtime.h>

#include "stemlib.h"
#include "stemutil.h"
#include "fileio_fftw3.h"
#include "qstem_gpu.h"

namespace {

void fail(const char* what) {
    fprintf(stderr, "qstem_gpu: %s: %s\n", what, qs_last_error());
    exit(1);
}

void check(int rc, const char* what) {
    if (rc != QS_OK) fail(what);
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        fprintf(stderr, "qstem_gpu: %s: %s\n", what, cudaGetErrorString(e));
        exit(1);
    }
}

// the MULS fields the library reads (libs/data_containers.h:103-308)
qs_params to_params(const MULS* m) {
    qs_params p;
    std::memset(&p, 0, sizeof p);
    p.mode = m->mode;
    p.nx = m->nx;
    p.ny = m->ny;
    p.potNx = m->potNx;
    p.potNy = m->potNy;
    p.slices = m->slices;
    p.cellDiv = m->cellDiv;
    p.outputInterval = m->outputInterval;
    p.centerSlices = m->centerSlices;
    p.nonPeriod = m->nonPeriod;
    p.nonPeriodZ = m->nonPeriodZ;
    p.potential3D = m->potential3D;
    p.fftpotential = m->fftpotential;
    p.bandlimittrans = m->bandlimittrans;
    p.tds = m->tds;
    p.resolutionX = m->resolutionX;
    p.resolutionY = m->resolutionY;
    p.sliceThickness = m->sliceThickness;
    p.czOffset = m->czOffset;
    p.potOffsetX = m->potOffsetX;
    p.potOffsetY = m->potOffsetY;
    p.potSizeX = m->potSizeX;
    p.potSizeY = m->potSizeY;
    p.ax = m->ax;
    p.by = m->by;
    p.c = m->c;
    p.atomRadius = m->atomRadius;
    p.v0 = m->v0;
    p.alpha = m->alpha;
    p.Cs = m->Cs;
    p.C5 = m->C5;
    p.df0 = m->df0;
    p.astigMag = m->astigMag;
    p.astigAngle = m->astigAngle;
    p.Cc = m->Cc;
    p.dE_E = m->dE_E;
    p.a33 = m->a33;
    p.a31 = m->a31;
    p.a44 = m->a44;
    p.a42 = m->a42;
    p.a55 = m->a55;
    p.a53 = m->a53;
    p.a51 = m->a51;
    p.a66 = m->a66;
    p.a64 = m->a64;
    p.a62 = m->a62;
    p.phi33 = m->phi33;
    p.phi31 = m->phi31;
    p.phi44 = m->phi44;
    p.phi42 = m->phi42;
    p.phi55 = m->phi55;
    p.phi53 = m->phi53;
    p.phi51 = m->phi51;
    p.phi66 = m->phi66;
    p.phi64 = m->phi64;
    p.phi62 = m->phi62;
    p.ismoth = m->ismoth;
    p.gaussFlag = m->gaussFlag;
    p.gaussScale = m->gaussScale;
    p.aAIS = m->aAIS;
    p.scanXStart = m->scanXStart;
    p.scanXStop = m->scanXStop;
    p.scanYStart = m->scanYStart;
    p.scanYStop = m->scanYStop;
    p.scanXN = m->scanXN;
    p.scanYN = m->scanYN;
    p.electronScale = m->electronScale;
    p.detectorNum = m->detectorNum;
    p.equalDivs = m->equalDivs;
    p.mulsRepeat1 = m->mulsRepeat1;
    p.mulsRepeat2 = m->mulsRepeat2;
    if (m->detectorNum > QS_MAX_DETECTORS) {
        fprintf(stderr, "qstem_gpu: at most %d detectors\n", QS_MAX_DETECTORS);
        exit(1);
    }
    for (int i = 0; i < m->detectorNum; i++) {
        const DetectorPtr& d = m->detectors[0][i];
        p.detectors[i].rInside = d->rInside;
        p.detectors[i].rOutside = d->rOutside;
        p.detectors[i].k2Inside = d->k2Inside;
        p.detectors[i].k2Outside = d->k2Outside;
        p.detectors[i].shiftX = d->shiftX;
        p.detectors[i].shiftY = d->shiftY;
    }
    return p;
}

void check_scope(const MULS* m) {
    if (m->mulsRepeat1 > 1) {
        fprintf(stderr, "qstem_gpu: this adapter runs each slab's stack once per pass (sequence m1 = 1); "
                        "repeated stacks run through qs_stem_run, qs_tem_run and qs_cbed_batch_run\n");
        exit(1);
    }
}

// the slice stack, built by make3DSlices and read by every thread
struct Stack {
    qs_ctx* ctx = nullptr;
    float* trans = nullptr;
    size_t cap = 0;
} g_stack;

// one context and its device buffers per calling thread
struct ThreadState {
    qs_ctx* ctx = nullptr;
    float *probe = nullptr, *det = nullptr, *dp = nullptr, *ew = nullptr;
    size_t nprobe = 0, ndet = 0, ndp = 0, new_ = 0;
    ~ThreadState() {
        if (!ctx) return;
        cudaFree(probe);
        cudaFree(det);
        cudaFree(dp);
        cudaFree(ew);
        qs_ctx_destroy(ctx);
    }
};
thread_local ThreadState t_state;

void grow(float** buf, size_t* cap, size_t floats) {
    if (*cap >= floats) return;
    cudaFree(*buf);
    *buf = nullptr;
    check_cuda(cudaMalloc(buf, sizeof(float) * floats), "device buffer");
    *cap = floats;
}

// the context of the calling thread, with room for one position: incident
// wave, detector values [nT][ndet], patterns and exit waves (one per
// thickness slot with `series`)
ThreadState& thread_state(const qs_params& p, int nT, int series) {
    ThreadState& s = t_state;
    if (!s.ctx) check(qs_ctx_create(0, &s.ctx), "context");
    const size_t N = (size_t)p.nx * p.ny, slots = series ? (size_t)nT : 1;
    grow(&s.probe, &s.nprobe, 2 * N);
    grow(&s.ew, &s.new_, 2 * N * slots);
    grow(&s.dp, &s.ndp, N * slots);
    grow(&s.det, &s.ndet, (size_t)nT * (p.detectorNum > 0 ? p.detectorNum : 1));
    return s;
}

}  // namespace

static void prepare_atoms(MULS* muls, atom* center);

void make3DSlices(MULS* muls, int nlayer, char* fileIn, atom* center) {
    static int divCount = 0;
    if (nlayer < 1) return;
    check_scope(muls);
    if (!g_stack.ctx) check(qs_ctx_create(0, &g_stack.ctx), "context");
    // the slab this call builds (stem3/stemlib.cpp:456-465, :709): slab 0
    // again and again for equal divisions
    if (divCount == 0 || muls->equalDivs) divCount = muls->cellDiv;
    divCount--;
    const int slab = muls->cellDiv - divCount - 1;
    if (divCount == muls->cellDiv - 1) {
        // the run's atoms (:467-488): read and displaced again for every run
        // after the first
        if (muls->avgCount != 0) {
            int natom = 0;
            muls->atoms = readUnitCell(&natom, fileIn, muls, 1);
            muls->natom = natom;
        }
        prepare_atoms(muls, center);
    }
    qs_params p = to_params(muls);
    const size_t floats = 2 * (size_t)p.slices * p.potNx * p.potNy;
    if (g_stack.cap < floats) {
        cudaFree(g_stack.trans);
        g_stack.trans = nullptr;
        check_cuda(cudaMalloc(&g_stack.trans, sizeof(float) * floats), "slice stack");
        g_stack.cap = floats;
    }
    // struct atom and qs_atom share one layout (libs/stemtypes_fftw3.h:70-77)
    check(qs_slab_build(g_stack.ctx, &p, (const qs_atom*)muls->atoms, muls->natom, slab, g_stack.trans, QS_SYNC),
          "slice build");
}

// centring, z order, configuration file and slice thicknesses of a run's
// atoms, as make3DSlices prepares them (stem3/stemlib.cpp:516-553, :603-626)
static void prepare_atoms(MULS* muls, atom* center) {
    atom* atoms = muls->atoms;
    const int natom = muls->natom;
    if (center != NULL) {
        const float_tt dx = muls->ax / 2.0f - center->x, dy = muls->by / 2.0f - center->y, dz = -center->z;
        for (int i = 0; i < natom; i++) {
            atoms[i].x += dx;
            if (atoms[i].x < 0.0f) atoms[i].x += muls->ax;
            else if (atoms[i].x > muls->ax) atoms[i].x -= muls->ax;
            atoms[i].y += dy;
            if (atoms[i].y < 0.0f) atoms[i].y += muls->by;
            else if (atoms[i].y > muls->by) atoms[i].y -= muls->by;
            atoms[i].z += dz;
            if (atoms[i].z < 0.0f) atoms[i].z += muls->c;
            else if (atoms[i].z > muls->c) atoms[i].z -= muls->c;
        }
    }
    // the z order the scatter-sum walks, and the configuration file (:540-553)
    qsort(atoms, natom, sizeof(atom), atomCompare);
    char buf[2048];
    snprintf(buf, sizeof buf, "%s/%s", muls->folder, muls->cfgFile);
    if (strlen(buf) >= 4 && strcmp(buf + strlen(buf) - 4, ".cfg") == 0) *(buf + strlen(buf) - 4) = '\0';
    if (muls->tds) snprintf(buf + strlen(buf), sizeof buf - strlen(buf), "_%d.cfg", muls->avgCount);
    else snprintf(buf + strlen(buf), sizeof buf - strlen(buf), ".cfg");
    writeCFG(atoms, natom, buf, muls);
    if (muls->cz == NULL) muls->cz = float1D(muls->slices, "cz");
    for (int i = 0; i < muls->slices; i++) muls->cz[i] = muls->sliceThickness;
}

void initSTEMSlices(MULS* muls, int nlayer) {
    // the phase grating and the band limit ran in make3DSlices
    (void)muls;
    (void)nlayer;
}

void probe(MULS* muls, WavePtr wave, double dx, double dy) {
    qs_params p = to_params(muls);
    ThreadState& s = t_state;
    if (!s.ctx) check(qs_ctx_create(0, &s.ctx), "context");
    check(qs_probe(s.ctx, &p, dx, dy, (float*)wave->wave[0], QS_HOST_IO), "probe");
}

int runMulsSTEM(MULS* muls, WavePtr wave) {
    check_scope(muls);
    if (!g_stack.trans) {
        fprintf(stderr, "qstem_gpu: runMulsSTEM before make3DSlices\n");
        exit(1);
    }
    // this pass: the current slab's stack once, a thickness slot after every
    // slice (slot l of slice l, the last slice in slot S), one position on a
    // 1 x 1 detector raster, the window at the wave's offsets
    const int S = muls->slices;
    qs_params p = to_params(muls);
    p.cellDiv = 1;
    p.mulsRepeat1 = p.mulsRepeat2 = 1;
    p.outputInterval = 1;
    p.scanXN = p.scanYN = 1;
    const int nL = qs_thickness_count(&p);  // S + 1
    // CBED at save level > 0 keeps the pattern of every thickness slot
    // (collectIntensity's diff_<t>.img, stem3/stemlib.cpp:2663-2676)
    const int series = (muls->mode == CBED && muls->saveLevel > 0) ? 1 : 0;
    ThreadState& s = thread_state(p, nL, series);
    const size_t N = (size_t)p.nx * p.ny;
    int ix = wave->iPosX, iy = wave->iPosY, zero = 0;
    qs_batch b = {1, &ix, &iy, &zero, &zero};
    check_cuda(cudaMemcpy(s.probe, wave->wave[0], sizeof(float) * 2 * N, cudaMemcpyHostToDevice), "incident wave");
    check(qs_multislice_run(s.ctx, &p, g_stack.trans, s.probe, &b, p.detectorNum > 0 ? s.det : NULL, s.dp, s.ew,
                            QS_SYNC | (series ? QS_SERIES : 0)),
          "multislice");
    check_cuda(cudaMemcpy(wave->wave[0], s.ew + (series ? 2 * N * (nL - 1) : 0), sizeof(float) * 2 * N,
                          cudaMemcpyDeviceToHost),
               "exit wave");
    check_cuda(cudaMemcpy(wave->diffpat[0], s.dp + (series ? N * (nL - 1) : 0), sizeof(float) * N,
                          cudaMemcpyDeviceToHost),
               "diffraction pattern");
    // slice l of this pass is slice totalSliceCount + l of the specimen;
    // collectIntensity files it under slot x / outputInterval, the
    // specimen's last slice under tCount (:2591-2610)
    const int SA = S * muls->cellDiv, tCount = (SA / muls->outputInterval);
    auto slot_of = [&](int l) {
        const int x = muls->totalSliceCount + l;
        return x < SA - 1 ? x / muls->outputInterval : tCount;
    };
    auto local_slot = [&](int l) { return l < S - 1 ? l : nL - 1; };
    if (p.detectorNum > 0) {
        // collectIntensity's detector semantics: a slot's pixel holds the
        // value of the slot's last slice, image2 its square
        std::vector<float> det((size_t)nL * p.detectorNum);
        check_cuda(cudaMemcpy(det.data(), s.det, sizeof(float) * det.size(), cudaMemcpyDeviceToHost), "detectors");
        for (int l = 0; l < S; l++) {
            const int t = slot_of(l), tl = local_slot(l);
            for (int i = 0; i < p.detectorNum; i++) {
                const float v = det[(size_t)tl * p.detectorNum + i];
                muls->detectors[t][i]->image[wave->detPosX][wave->detPosY] = v;
                muls->detectors[t][i]->image2[wave->detPosX][wave->detPosY] = v * v;
            }
        }
    }
    if (series) {
        // each slot's pattern is that of its last slice in this pass
        std::vector<int> last(tCount + 1, -1);
        for (int l = 0; l < S; l++) last[slot_of(l)] = l;
        std::vector<float> pat(N), fin(N);
        std::memcpy(fin.data(), wave->diffpat[0], sizeof(float) * N);
        char name[1100];
        for (int t = 0; t <= tCount; t++) {
            if (last[t] < 0) continue;
            check_cuda(cudaMemcpy(pat.data(), s.dp + N * local_slot(last[t]), sizeof(float) * N,
                                  cudaMemcpyDeviceToHost),
                       "patterns");
            std::memcpy(wave->diffpat[0], pat.data(), sizeof(float) * N);
            snprintf(name, sizeof name, "%s/diff_%d.img", muls->folder, t);
            if (muls->avgCount == 0) {
                wave->WriteDiffPat(name);
            } else {
                wave->ReadAvgArray(name);
                for (size_t k = 0; k < N; k++)
                    wave->avgArray[0][k] = (muls->avgCount * wave->avgArray[0][k] + pat[k]) / (muls->avgCount + 1);
                wave->WriteAvgArray(name);
            }
        }
        std::memcpy(wave->diffpat[0], fin.data(), sizeof(float) * N);
    }
    // the exit wave's intensity (:2497-2518)
    double sum = 0.0;
    const float* w = (const float*)wave->wave[0];
    for (size_t k = 0; k < N; k++) sum += (double)w[2 * k] * w[2 * k] + (double)w[2 * k + 1] * w[2 * k + 1];
    wave->intIntensity = (float_tt)(sum / (double)N);
    if (muls->saveFlag && (muls->saveLevel > 1 || muls->cellDiv > 1)) wave->WriteWave(wave->fileout);
    return 0;
}

void collectIntensity(MULS* muls, WavePtr wave, int slice) {
    qs_params p = to_params(muls);
    ThreadState& s = t_state;
    if (!s.ctx) check(qs_ctx_create(0, &s.ctx), "context");
    double sums[QS_MAX_DETECTORS];
    check(qs_collect(s.ctx, &p, (const float*)wave->wave[0], sums, (float*)wave->diffpat[0], QS_HOST_IO),
          "collectIntensity");
    // the thickness slot of `slice` (:2591-2610)
    const int tCount = qs_thickness_count(&p) - 1;
    const int t = (slice < muls->slices * muls->cellDiv - 1) ? slice / muls->outputInterval : tCount;
    const double scale = muls->electronScale / ((double)(p.nx * p.ny) * (double)(p.nx * p.ny));
    for (int i = 0; i < p.detectorNum; i++) {
        const float v = (float)(sums[i] * scale);
        muls->detectors[t][i]->image[wave->detPosX][wave->detPosY] = v;
        muls->detectors[t][i]->image2[wave->detPosX][wave->detPosY] = v * v;
    }
}
