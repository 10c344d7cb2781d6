/* Single-process stand-in for the Global Arrays C++ API, just large enough for
 * the reference's compute sources (PsociConfigs.C, PsociDeterminants.C,
 * PsociIntegrals.C, PsociHamiltonian.C, PsociTimer.C) to compile and run as
 * one rank.  Collectives are no-ops, node id is 0, node count is 1.
 * Test infrastructure only: used to build the reference oracle under oracle/_ref.
 */
#ifndef PSOCI_REF_SHIM_GAXX_H
#define PSOCI_REF_SHIM_GAXX_H
#include <cstdio>
#include <cstdlib>
#include "ga.h"

namespace GA {
inline int nodeid() { return 0; }
inline int nodes() { return 1; }
inline void Terminate() { std::fprintf(stderr, "ref shim: GA::Terminate\n"); std::abort(); }
inline void error(const char *msg, int code) {
  std::fprintf(stderr, "ref shim: GA::error %s (%d)\n", msg, code);
  std::abort();
}
inline void sync() {}
inline void brdcst(void *, int, int) {}
inline void igop(int *, int, char *) {}
inline void igop(long *, int, char *) {}
inline void gop(double *, int, char *) {}
struct Services { void sync() {} };
static Services SERVICES;

class GlobalArray {
 public:
  void checkHandle(const char *) {}
  void checkHandle(char *) {}
  void destroy() {}
  void zero() {}
  void printDistribution() {}
  void distribution(int, int *lo, int *hi) { lo[0] = lo[1] = 0; hi[0] = hi[1] = -1; }
  void get(int *, int *, void *, int *) { Terminate(); }
  void put(int *, int *, void *, int *) { Terminate(); }
};
inline GlobalArray *createGA(int, int, int *, char *, int *) { return new GlobalArray(); }
}  // namespace GA
#endif
