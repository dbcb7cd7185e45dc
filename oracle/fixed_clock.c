/*
 * fixed_clock.c -- a settable clock for the reference's time-seeded
 * generators.  TEST INFRASTRUCTURE ONLY, linked into oracle/_ref's programs.
 *
 * The reference seeds its thermal displacements and CBED source offsets
 * with -(long)time(NULL) (libs/fileio_fftw3.cpp:496, stem3/stem3.cpp:2065).
 * This definition of time() takes precedence over the C library's in the
 * programs it is linked into: with QS_REF_CLOCK set it returns that value,
 * so a reference run draws a known sequence; otherwise the real clock.
 */
#include <stdlib.h>
#include <time.h>

time_t time(time_t *tloc) {
    const char *fixed = getenv("QS_REF_CLOCK");
    time_t now;
    if (fixed && *fixed) {
        now = (time_t)strtoll(fixed, NULL, 10);
    } else {
        struct timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        now = ts.tv_sec;
    }
    if (tloc) *tloc = now;
    return now;
}
