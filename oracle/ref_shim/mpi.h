/* Single-process stand-in for the two MPI names the reference timer uses.
 * Test infrastructure only. */
#ifndef PSOCI_REF_SHIM_MPI_H
#define PSOCI_REF_SHIM_MPI_H
#include <sys/time.h>
typedef int MPI_Comm;
static inline double MPI_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, 0);
  return tv.tv_sec + 1e-6 * tv.tv_usec;
}
#endif
