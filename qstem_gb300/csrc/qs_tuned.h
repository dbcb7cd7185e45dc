// qs_tuned.h -- launch schedules picked by measurement (qstem_gb300/tune.py).
//
// QS_ROW_MIN_BLOCKS_<N>: CTAs per SM the row pass ms_rows<N, *> is compiled
// for (its __launch_bounds__ minimum, i.e. the register budget per thread);
// 1 leaves the compiler unconstrained.  tune.py rebuilds the row pass with
// each candidate for every line length at once, times the row pass of each
// size on the GPU with the library's CUDA-event counters (random slice stack,
// 8 slices, 128-1024 waves) and writes the fastest here.  Any value can be
// overridden with -D at build time.
//
// Measured on GB300 (us per position-slice, row pass):
//   N     1      2      3      4      5      6      8
//   256   0.195  -      -      0.200  -      0.184  0.180
//   384   0.773  -      0.714  0.734  0.806  0.808  -
//   512   -      -      0.848  -      -      -      -
//   768   3.47   3.37   3.40   4.25   -      -      -
//   1024  4.86   3.56   5.21   8.22   -      -      -
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
#define QS_ROW_MIN_BLOCKS_768 2
#endif
#ifndef QS_ROW_MIN_BLOCKS_1024
#define QS_ROW_MIN_BLOCKS_1024 2
#endif
