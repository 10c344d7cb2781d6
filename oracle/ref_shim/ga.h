/* Single-process stand-in for the Global Arrays C API constants used by the
 * reference compute sources.  Test infrastructure only. */
#ifndef PSOCI_REF_SHIM_GA_H
#define PSOCI_REF_SHIM_GA_H
#define C_INT 1
#define C_LONG 2
#define C_DBL 3
#include <sys/time.h>
static inline double GA_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, 0);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}
#endif
