// qs_tuned.h -- launch schedules picked by measurement (qstem_gb300/tune.py).
//
// QS_ROW_MIN_BLOCKS_<N>: CTAs per SM the row pass ms_rows<N, *> is compiled
// for (its __launch_bounds__ minimum, i.e. the register budget per thread;
// 1 allows up to 255 registers).  tune.py rebuilds the row pass with
// each candidate for every line length at once, times the row pass of each
// size on the GPU with the library's CUDA-event counters (random slice stack,
// 8 slices, 128-1024 waves) and writes the fastest here.  Any value can be
// overridden with -D at build time.
//
// The tables below began as the output of
//   python -m qstem_gb300.tune --write
// (candidates 1,2,3,4,6,8, row shapes of 4 and 8 lines, sizes 256-1024) on
// GB300: phase 0 picked the factorisations and column tiles, phase 1 the
// row-pass shapes and the budgets of both passes, phase 2 the row adjoint's
// budget (it prints the whole sweep).  For the column pass a stated 1 (the
// compiler may use up to 255 registers) differs from leaving the bound open.
// Later changes were each timed side by side against the tables of the day
// (python -m qstem_gb300.tune --compare ...), in this order:
//  - after the column tiles became 16-byte copies of column pairs: tiles,
//    stages and budgets 256 8 columns x 2 stages at 4 CTAs per SM, 512 16 x 1
//    at 2;
//  - 768-point lines as 16 threads x 48 elements (radices 48 x 16, two
//    passes): rows 2.49 -> 2.37 us, columns 1.90 -> 1.81 us per
//    position-slice; 384-point column lines as 8 x 48 (48 x 8): 0.414 ->
//    0.386;
//  - packed two-lane additions (QS_PACKED_*, below);
//  - then the 768 row pass at 3 CTAs per SM (2.25 -> 1.92 us; budgets 4 and 5
//    at 384/512/1024 and 3 at 1024 measured slower), 384-point rows as
//    8 x 48 with 16 lines a CTA at 3 CTAs per SM (0.578 -> 0.554 us), and
//    one-stage 16-column tiles at 768 (2 CTAs per SM; 1.667 -> 1.502 us) and
//    384 (3 CTAs per SM; 0.370 -> 0.356).
// The tuner sweeps budgets, row shapes, factorisations and tiles; the thread
// layouts (QS_LINE_T_*, QS_COL_LINE_T_*) and the packing bits are set here
// from the side-by-side timings.
#pragma once

#ifndef QS_ROW_MIN_BLOCKS_64
#define QS_ROW_MIN_BLOCKS_64 1
#endif
#ifndef QS_ROW_MIN_BLOCKS_128
#define QS_ROW_MIN_BLOCKS_128 1
#endif
#ifndef QS_ROW_MIN_BLOCKS_256
#define QS_ROW_MIN_BLOCKS_256 8
#endif
#ifndef QS_ROW_MIN_BLOCKS_384
#define QS_ROW_MIN_BLOCKS_384 3
#endif
#ifndef QS_ROW_MIN_BLOCKS_512
#define QS_ROW_MIN_BLOCKS_512 3
#endif
#ifndef QS_ROW_MIN_BLOCKS_768
#define QS_ROW_MIN_BLOCKS_768 3
#endif
#ifndef QS_ROW_MIN_BLOCKS_1024
#define QS_ROW_MIN_BLOCKS_1024 4
#endif
#ifndef QS_COL_MIN_BLOCKS_64
#define QS_COL_MIN_BLOCKS_64 1
#endif
#ifndef QS_COL_MIN_BLOCKS_128
#define QS_COL_MIN_BLOCKS_128 1
#endif
#ifndef QS_COL_MIN_BLOCKS_256
#define QS_COL_MIN_BLOCKS_256 4
#endif
#ifndef QS_COL_MIN_BLOCKS_384
#define QS_COL_MIN_BLOCKS_384 3
#endif
#ifndef QS_COL_MIN_BLOCKS_512
#define QS_COL_MIN_BLOCKS_512 2
#endif
#ifndef QS_COL_MIN_BLOCKS_768
#define QS_COL_MIN_BLOCKS_768 2
#endif
#ifndef QS_COL_MIN_BLOCKS_1024
#define QS_COL_MIN_BLOCKS_1024 2
#endif
#ifndef QS_ADJ_MIN_BLOCKS_64
#define QS_ADJ_MIN_BLOCKS_64 1
#endif
#ifndef QS_ADJ_MIN_BLOCKS_128
#define QS_ADJ_MIN_BLOCKS_128 1
#endif
#ifndef QS_ADJ_MIN_BLOCKS_256
#define QS_ADJ_MIN_BLOCKS_256 4
#endif
#ifndef QS_ADJ_MIN_BLOCKS_384
#define QS_ADJ_MIN_BLOCKS_384 3
#endif
#ifndef QS_ADJ_MIN_BLOCKS_512
#define QS_ADJ_MIN_BLOCKS_512 3
#endif
#ifndef QS_ADJ_MIN_BLOCKS_768
#define QS_ADJ_MIN_BLOCKS_768 2
#endif
#ifndef QS_ADJ_MIN_BLOCKS_1024
#define QS_ADJ_MIN_BLOCKS_1024 1
#endif
#ifndef QS_ROW_LINES_64
#define QS_ROW_LINES_64 8
#endif
#ifndef QS_ROW_LINES_128
#define QS_ROW_LINES_128 8
#endif
#ifndef QS_ROW_LINES_256
#define QS_ROW_LINES_256 8
#endif
#ifndef QS_ROW_LINES_384
#define QS_ROW_LINES_384 16
#endif
#ifndef QS_ROW_LINES_512
#define QS_ROW_LINES_512 8
#endif
#ifndef QS_ROW_LINES_768
#define QS_ROW_LINES_768 8
#endif
#ifndef QS_ROW_LINES_1024
#define QS_ROW_LINES_1024 4
#endif

// QS_COL_TILE_<N>: columns per column-pass tile (8 or 16; with two stages
// the 16-column tile fits in shared memory only up to 768).
#ifndef QS_COL_TILE_64
#define QS_COL_TILE_64 16
#endif
#ifndef QS_COL_TILE_128
#define QS_COL_TILE_128 16
#endif
#ifndef QS_COL_TILE_256
#define QS_COL_TILE_256 8
#endif
#ifndef QS_COL_TILE_384
#define QS_COL_TILE_384 16
#endif
#ifndef QS_COL_TILE_512
#define QS_COL_TILE_512 16
#endif
#ifndef QS_COL_TILE_768
#define QS_COL_TILE_768 16
#endif
#ifndef QS_COL_TILE_1024
#define QS_COL_TILE_1024 8
#endif

// QS_COL_STAGES_<N>: shared-memory tile stages of the column pass: 2 copies
// the next tile with cp.async while one is transformed, 1 leaves the overlap
// to other CTAs (half the shared memory per CTA).
#ifndef QS_COL_STAGES_64
#define QS_COL_STAGES_64 2
#endif
#ifndef QS_COL_STAGES_128
#define QS_COL_STAGES_128 2
#endif
#ifndef QS_COL_STAGES_256
#define QS_COL_STAGES_256 2
#endif
#ifndef QS_COL_STAGES_384
#define QS_COL_STAGES_384 1
#endif
#ifndef QS_COL_STAGES_512
#define QS_COL_STAGES_512 1
#endif
#ifndef QS_COL_STAGES_768
#define QS_COL_STAGES_768 1
#endif
#ifndef QS_COL_STAGES_1024
#define QS_COL_STAGES_1024 1
#endif

// QS_LINE_T_384, QS_LINE_T_768: threads per row line of the 384- and
// 768-point transforms: 16 and 32 hold 24 elements a thread (three radix
// passes), 8 and 16 hold 48 (the two-pass factorisations 8x48 / 48x8 and
// 16x48 / 48x16, entries 5 and 6 of the lists).
#ifndef QS_LINE_T_384
#define QS_LINE_T_384 8
#endif
#ifndef QS_LINE_T_768
#define QS_LINE_T_768 16
#endif
// QS_COL_LINE_T_<N>: the same for the column lines (default: the rows')
#ifndef QS_COL_LINE_T_384
#define QS_COL_LINE_T_384 QS_LINE_T_384
#endif
#ifndef QS_COL_LINE_T_768
#define QS_COL_LINE_T_768 QS_LINE_T_768
#endif

// QS_RADIX_ROW_<N>, QS_RADIX_COL_<N>: which factorisation of the row and of
// the column line transform (the lists of Line / LineCol in qs_fft.cuh;
// 0 = the first).  Every translation unit must be compiled with the same
// choice (the twiddle tables follow it).
#ifndef QS_RADIX_ROW_384
#define QS_RADIX_ROW_384 6
#endif
#ifndef QS_RADIX_ROW_512
#define QS_RADIX_ROW_512 0
#endif
#ifndef QS_RADIX_ROW_768
#define QS_RADIX_ROW_768 6
#endif
#ifndef QS_RADIX_ROW_1024
#define QS_RADIX_ROW_1024 0
#endif
#ifndef QS_RADIX_COL_384
#define QS_RADIX_COL_384 6
#endif
#ifndef QS_RADIX_COL_512
#define QS_RADIX_COL_512 0
#endif
#ifndef QS_RADIX_COL_768
#define QS_RADIX_COL_768 6
#endif
#ifndef QS_RADIX_COL_1024
#define QS_RADIX_COL_1024 0
#endif

// QS_PACKED_ROWS, QS_PACKED_COLS_<N>: the butterflies' complex additions of
// the 384- to 1024-point row / column transforms as packed two-lane float
// instructions (add/sub.rn.f32x2; results bit-identical): bit 0 the forward,
// bit 1 the inverse transform.  Measured: rows packed both ways 14.5 % faster
// at 512 points, 12 % at 1024, 5 % at 768 and 4 % at 384; column passes with
// the forward transform packed 4 % faster at 512, 8 % at 768, 3.6 % at 384,
// 1.7 % at 1024 (the inverse packed as well: slower at 512 and 1024).
#ifndef QS_PACKED_ROWS
#define QS_PACKED_ROWS 3
#endif
#ifndef QS_PACKED_COLS_384
#define QS_PACKED_COLS_384 1
#endif
#ifndef QS_PACKED_COLS_512
#define QS_PACKED_COLS_512 1
#endif
#ifndef QS_PACKED_COLS_768
#define QS_PACKED_COLS_768 1
#endif
#ifndef QS_PACKED_COLS_1024
#define QS_PACKED_COLS_1024 1
#endif
// the 256-point lines (rows and columns share one configuration; forward,
// inverse or both packed measured within 1 % of scalar additions)
#ifndef QS_PACKED_256
#define QS_PACKED_256 0
#endif
