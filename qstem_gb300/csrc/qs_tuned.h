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
// The tables below are the output of
//   python -m qstem_gb300.tune --candidates 1,2,3,4,6,8 --lines 4,8 --sizes 256,384,512,768,1024
// (the row adjoint's 5 at 256^2 from a sweep with 5 among the candidates)
// on GB300 (it prints the whole sweep).  For the column pass a stated 1 (the compiler may use up to 255 registers) differs
// from leaving the bound open, and measured faster at 384^2 and 768^2.
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
#define QS_COL_MIN_BLOCKS_256 2
#endif
#ifndef QS_COL_MIN_BLOCKS_384
#define QS_COL_MIN_BLOCKS_384 1
#endif
#ifndef QS_COL_MIN_BLOCKS_512
#define QS_COL_MIN_BLOCKS_512 2
#endif
#ifndef QS_COL_MIN_BLOCKS_768
#define QS_COL_MIN_BLOCKS_768 1
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
#define QS_ADJ_MIN_BLOCKS_256 5
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
#define QS_ROW_LINES_384 8
#endif
#ifndef QS_ROW_LINES_512
#define QS_ROW_LINES_512 8
#endif
#ifndef QS_ROW_LINES_768
#define QS_ROW_LINES_768 4
#endif
#ifndef QS_ROW_LINES_1024
#define QS_ROW_LINES_1024 4
#endif
