/*
 * ref_harness.cpp -- drives the reference's own CPU path and dumps its
 * intermediate and final arrays as raw little-endian binaries.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile against the reference
 * sources where they lie (stem3/*.cpp, libs/*.cpp, compiled unmodified, with
 * stem3.cpp's main renamed) and the FFT shim; used to pin the C restatement
 * (qs_oracle.c) and to generate the committed golden fixtures.  It calls, in
 * the order stem3's main does (stem3/stem3.cpp:111-170):
 *   parOpen + readFile                 stem3/stem3.cpp:133-139, :612
 *   make3DSlices                       stem3/stemlib.cpp:383
 *   getAtomPotential3D / Offset3D      stem3/stemlib.cpp:1342, :1548
 *   initSTEMSlices                     stem3/stemlib.cpp:2199
 *   probe                              stem3/stemlib.cpp:1952
 *   doSTEM / doCBED / doTEM            stem3/stem3.cpp:2722, :2048, :2354
 * and writes:
 *   meta.txt              key = value lines of the MULS fields the hot path reads
 *   atoms.bin             readFile's atoms (struct atom, 28 bytes each)
 *   atoms_sorted.bin      the same after make3DSlices sorted them by z
 *   potential.bin         trans[slices][potNx][potNy] (complex float) after make3DSlices
 *   lut_<Z>.bin / lutq_<Z>.bin   LUTs (Nz_lut x Nr complex float)
 *   trans.bin             after initSTEMSlices
 *   probe.bin             probe(muls, wave, nx/2*dx, ny/2*dy)
 *   det_<t>_<i>.bin       detector images (scanXN x scanYN float) after doSTEM
 * Usage: ref_harness <file.qsc> <outdir> [run]
 */
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "data_containers.h"
#include "readparams.h"
#include "stemlib.h"
#include "stemutil.h"
#include "customslice.h"

extern MULS muls;
void readFile();
void displayParams();
void doSTEM();
void doCBED();
void doTEM();

static std::string g_out;

static void dump(const char *name, const void *p, size_t bytes) {
    std::string path = g_out + "/" + name;
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    fwrite(p, 1, bytes, f);
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: ref_harness file.qsc outdir [run]\n");
        return 2;
    }
    g_out = argv[2];
    const bool run = (argc > 3) && strcmp(argv[3], "run") == 0;
    muls.nCellX = 1; muls.nCellY = 1; muls.nCellZ = 1;
    if (parOpen(argv[1]) == 0) { fprintf(stderr, "cannot open %s\n", argv[1]); return 2; }
    readFile();
    displayParams();
    if (muls.mode == 1 /* STEM */) {
        for (muls.avgCount = 0; muls.avgCount < muls.avgRuns; muls.avgCount++)
            muls.dE_E = muls.dE_EArray[muls.avgCount];
        muls.showProbe = 0;
        muls.avgCount = -1;
    }

    dump("atoms.bin", muls.atoms, sizeof(atom) * (size_t)muls.natom);

    /* make3DSlicesFT clears trans with sizeof(fftw_complex) (16 bytes) per
     * element of its fftwf_complex (8-byte) array, writing past the end of
     * the array readFile allocated (stem3/customslice.cpp:251, against
     * stem3/stem3.cpp:1532).  For custom scattering factors the harness
     * hands it a stack of twice the slices, so that the clearing stays in
     * memory it owns; the slices it fills are the first half, unchanged.
     * (The potential-array FFT plans stay on readFile's array: the band
     * limit that uses them is off in these runs.) */
    if (muls.scatFactor == CUSTOM)
        muls.trans = complex3Df(2 * muls.slices, muls.potNx, muls.potNy, "trans");

    /* The reference builds the slices and phase gratings once per run inside
     * doSTEM; here the same calls are made once beforehand so that their
     * outputs can be captured (they are repeated identically inside the run). */
    int saveAvg = muls.avgCount;
    muls.avgCount = 0;
    if (muls.scatFactor == CUSTOM) /* doCBED's custom scattering factors (stem3/stem3.cpp:2177) */
        make3DSlicesFT(&muls);
    else
        make3DSlices(&muls, muls.slices, muls.atomPosFile, NULL);
    dump("atoms_sorted.bin", muls.atoms, sizeof(atom) * (size_t)muls.natom);
    size_t ntrans = (size_t)muls.slices * muls.potNx * muls.potNy;
    dump("potential.bin", muls.trans[0][0], ntrans * sizeof(fftwf_complex));

    for (int k = 0; k < muls.atomKinds; k++) {
        int Z = muls.Znums[k];
        int nzSub = 0, Nr = 0, Nz = 0;
        /* B is ignored after the first call (static state, stemlib.cpp:1362) */
        fftwf_complex *lut = getAtomPotential3D(Z, &muls, 0.0, &nzSub, &Nr, &Nz);
        char nm[64];
        snprintf(nm, sizeof nm, "lut_%d.bin", Z);
        dump(nm, lut, sizeof(fftwf_complex) * (size_t)Nr * Nz);
        fftwf_complex *lutq = getAtomPotentialOffset3D(Z, &muls, 0.0, &nzSub, &Nr, &Nz, 1.0f);
        if (lutq) {
            snprintf(nm, sizeof nm, "lutq_%d.bin", Z);
            dump(nm, lutq, sizeof(fftwf_complex) * (size_t)Nr * Nz);
        }
        FILE *f = fopen((g_out + "/lut_dims.txt").c_str(), k ? "a" : "w");
        fprintf(f, "%d %d %d %d\n", Z, Nz, Nr, nzSub);
        fclose(f);
    }

    if (!muls.potential3D) {
        /* the 2-D tables make3DSlices used (cached by Z after their first
         * call, stem3/stemlib.cpp:1750-1857) */
        const int nx2 = 2 * 2 * (int)ceil(muls.atomRadius / muls.resolutionX);
        const int ny2 = 2 * 2 * (int)ceil(muls.atomRadius / muls.resolutionY);
        for (int k = 0; k < muls.atomKinds; k++) {
            int Z = muls.Znums[k];
            fftwf_complex *l2 = getAtomPotential2D(Z, &muls, 0.0);
            char nm[64];
            snprintf(nm, sizeof nm, "lut2d_%d.bin", Z);
            dump(nm, l2, sizeof(fftwf_complex) * (size_t)nx2 * ny2);
            FILE *f = fopen((g_out + "/lut2d_dims.txt").c_str(), k ? "a" : "w");
            fprintf(f, "%d %d %d\n", Z, nx2, ny2);
            fclose(f);
        }
    }

    initSTEMSlices(&muls, muls.slices);
    dump("trans.bin", muls.trans[0][0], ntrans * sizeof(fftwf_complex));

    /* A cell divided into unequal slabs: make3DSlices builds slab k on its
     * k-th call (a static counter, stem3/stemlib.cpp:456-465).  Capture the
     * other slabs too; after cellDiv calls the counter is back where doSTEM
     * expects it, so its first call builds slab 0 again. */
    if (muls.cellDiv > 1 && !muls.equalDivs) {
        for (int k = 1; k < muls.cellDiv; k++) {
            char nm[64];
            make3DSlices(&muls, muls.slices, muls.atomPosFile, NULL);
            snprintf(nm, sizeof nm, "potential_%d.bin", k);
            dump(nm, muls.trans[0][0], ntrans * sizeof(fftwf_complex));
            initSTEMSlices(&muls, muls.slices);
            snprintf(nm, sizeof nm, "trans_%d.bin", k);
            dump(nm, muls.trans[0][0], ntrans * sizeof(fftwf_complex));
        }
    }

    {
        WavePtr wave = WavePtr(new WAVEFUNC(muls.nx, muls.ny, muls.resolutionX, muls.resolutionY));
        probe(&muls, wave, muls.nx / 2 * muls.resolutionX, muls.ny / 2 * muls.resolutionY);
        dump("probe.bin", wave->wave[0], sizeof(fftwf_complex) * (size_t)muls.nx * muls.ny);
    }
    muls.avgCount = saveAvg;

    FILE *m = fopen((g_out + "/meta.txt").c_str(), "w");
    fprintf(m, "mode = %d\nnx = %d\nny = %d\npotNx = %d\npotNy = %d\nslices = %d\n", muls.mode,
            muls.nx, muls.ny, muls.potNx, muls.potNy, muls.slices);
    fprintf(m, "natom = %d\nresolutionX = %.9g\nresolutionY = %.9g\n", muls.natom,
            muls.resolutionX, muls.resolutionY);
    fprintf(m, "sliceThickness = %.9g\nczOffset = %.9g\nax = %.9g\nby = %.9g\nc = %.9g\n",
            muls.sliceThickness, muls.czOffset, muls.ax, muls.by, muls.c);
    fprintf(m, "potOffsetX = %.9g\npotOffsetY = %.9g\npotSizeX = %.9g\npotSizeY = %.9g\n",
            muls.potOffsetX, muls.potOffsetY, muls.potSizeX, muls.potSizeY);
    fprintf(m, "scanXStart = %.9g\nscanXStop = %.9g\nscanXN = %d\n", muls.scanXStart,
            muls.scanXStop, muls.scanXN);
    fprintf(m, "scanYStart = %.9g\nscanYStop = %.9g\nscanYN = %d\n", muls.scanYStart,
            muls.scanYStop, muls.scanYN);
    fprintf(m, "v0 = %.9g\nalpha = %.9g\nCs = %.9g\nC5 = %.9g\ndf0 = %.9g\n", muls.v0,
            muls.alpha, muls.Cs, muls.C5, muls.df0);
    fprintf(m, "electronScale = %.9g\noutputInterval = %d\ncellDiv = %d\nequalDivs = %d\n", muls.electronScale,
            muls.outputInterval, muls.cellDiv, muls.equalDivs);
    fprintf(m, "astigMag = %.9g\nastigAngle = %.9g\na33 = %.9g\nphi33 = %.9g\nCc = %.9g\n",
            muls.astigMag, muls.astigAngle, muls.a33, muls.phi33, muls.Cc);
    fprintf(m, "aAIS = %.9g\ngaussFlag = %d\ngaussScale = %.9g\navgRuns = %d\n", muls.aAIS,
            muls.gaussFlag, muls.gaussScale, muls.avgRuns);
    fprintf(m, "atomRadius = %.9g\nnonPeriod = %d\nnonPeriodZ = %d\ncenterSlices = %d\n",
            muls.atomRadius, muls.nonPeriod, muls.nonPeriodZ, muls.centerSlices);
    fprintf(m, "bandlimittrans = %d\ntds = %d\nismoth = %d\ndetectorNum = %d\n",
            muls.bandlimittrans, muls.tds, muls.ismoth, muls.detectorNum);
    for (int i = 0; i < muls.detectorNum && !muls.detectors.empty(); i++)
        fprintf(m, "det%d = %.9g %.9g %.9g %.9g %.9g %.9g\n", i, muls.detectors[0][i]->rInside,
                muls.detectors[0][i]->rOutside, muls.detectors[0][i]->k2Inside,
                muls.detectors[0][i]->k2Outside, muls.detectors[0][i]->shiftX,
                muls.detectors[0][i]->shiftY);
    fclose(m);

    if (!run) return 0;
    try {
        if (muls.mode == 1) doSTEM();
        else if (muls.mode == 2) doCBED();
        else if (muls.mode == 3) doTEM();
    } catch (const std::exception &e) {
        /* doTEM reads a diff.img it never writes (stem3/stem3.cpp:2545-2547) */
        FILE *f = fopen((g_out + "/exception.txt").c_str(), "w");
        fprintf(f, "%s\n", e.what());
        fclose(f);
    }
    if (muls.mode == 1) {
        int tCount = (int)muls.detectors.size();
        for (int t = 0; t < tCount; t++)
            for (int i = 0; i < muls.detectorNum; i++) {
                char nm[64];
                snprintf(nm, sizeof nm, "det_%d_%d.bin", t, i);
                dump(nm, muls.detectors[t][i]->image[0],
                     sizeof(float) * (size_t)muls.scanXN * muls.scanYN);
            }
    }
    return 0;
}
