// Serial stand-ins for the few MPI names the reference's headers use outside
// its USE_MPI branches (include/grid_ghosts.hh:56-76, a branch taken only for
// distributed grids).  Force-included (-include) into the reference's
// translation units by oracle/ref/Makefile; the build itself is the
// reference's single-process (non-MPI) configuration.  Test infrastructure
// for oracle/_ref.
#pragma once
#if !defined(USE_MPI)
#include <cstring>

namespace MPI {
inline int get_size(void) { return 1; }
inline int get_rank(void) { return 0; }
}  // namespace MPI

#define MPI_LONG_LONG 0
#define MPI_COMM_WORLD 0
// one task: every gather returns the caller's own block
inline int MPI_Allgather(const void* send, int count, int, void* recv, int, int, int) {
  std::memcpy(recv, send, (size_t)count * sizeof(long long));
  return 0;
}
#endif
