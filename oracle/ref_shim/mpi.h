// TEST INFRASTRUCTURE: single-rank stand-in for the MPI calls PeriDEM's driver and time
// loop make (run/simulate3d.cpp:59-63,149; src/particle/timeloop.h:236-237,658,815,861-875).
// With one rank MPI_Allreduce(MPI_IN_PLACE, ..., MPI_SUM) is the identity and the
// connectivity send/receive paths are never taken.
#ifndef PD_SHIM_MPI_H
#define PD_SHIM_MPI_H
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct {
  int count;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_UNSIGNED 2
#define MPI_SUM 1
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_MAX_PROCESSOR_NAME 64

inline int MPI_Init(int *, char ***) { return 0; }
inline int MPI_Finalize() { return 0; }
inline int MPI_Comm_size(MPI_Comm, int *n) {
  *n = 1;
  return 0;
}
inline int MPI_Comm_rank(MPI_Comm, int *r) {
  *r = 0;
  return 0;
}
inline int MPI_Get_processor_name(char *name, int *len) {
  std::strcpy(name, "local");
  *len = 5;
  return 0;
}
inline int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
inline int MPI_Probe(int, int, MPI_Comm, MPI_Status *s) {
  if (s) s->count = 0;
  return 0;
}
inline int MPI_Get_count(const MPI_Status *s, MPI_Datatype, int *c) {
  *c = s ? s->count : 0;
  return 0;
}
inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) { return 0; }
inline int MPI_Barrier(MPI_Comm) { return 0; }
#endif
