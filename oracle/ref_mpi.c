/* ref_mpi.c -- single-host stand-in for the MPI calls of the reference
 * programs, and the main() of every program translated by oracle/ref_f90c.py.
 *
 * TEST INFRASTRUCTURE ONLY: it runs translated reference programs to pin
 * the oracle. It is not part of the product.
 *
 * Each MPI rank is a forked process. The ranks meet at a process-shared
 * pthread barrier placed in anonymous shared memory, next to one mailbox per
 * rank. Only the calls that seismic_CPML_3D_isotropic_MPI_OpenMP.f90 makes
 * are provided:
 *   - MPI_INIT, MPI_FINALIZE, MPI_COMM_SIZE, MPI_COMM_RANK, MPI_BARRIER;
 *   - MPI_SENDRECV, for the shift exchanges of 3D:811-823 and 951-963, in
 *     which every rank sends to at most one rank and receives from at most
 *     one. A receive checks that its message came from the named source
 *     and has the named length;
 *   - MPI_REDUCE and MPI_ALLREDUCE with SUM, MAX and MIN, for 3D:1179-1186.
 *     The root combines the contributions in rank order 0, 1, ..., n-1.
 *     MPI leaves that order to the implementation, so pins on a reduced sum
 *     use a tolerance.
 * Every call is collective, as in the reference, which calls each of them
 * on all ranks in the same order. The numbers behind the mpif.h constants
 * match MPIF_PARAMETERS in ref_f90c.py.
 *
 * Usage: <program> [-np N] [-o outdir] [-t seconds]. The parent waits for
 * the ranks. If one fails, or the time limit passes, it kills the rest and
 * exits non-zero.
 */
#define _GNU_SOURCE
#include <errno.h>
#include <pthread.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

void ref_main(void);
extern const long ref_message_capacity; /* elements of the largest array */

enum { T_DOUBLE = 1, T_INTEGER = 2 };
enum { OP_SUM = 1, OP_MAX = 2, OP_MIN = 3 };
enum { PROC_NULL = -2, MAX_PROCS = 256, MAX_REDUCE = 64 };

typedef struct {
  pthread_barrier_t barrier;
  int from[MAX_PROCS];
  long bytes[MAX_PROCS];
  double reduce[MAX_PROCS][MAX_REDUCE];
} shared_t;

static int g_rank = 0, g_size = 1;
static const char* g_outdir = ".";
static shared_t* g_sh = NULL;
static unsigned char* g_box = NULL; /* g_size mailboxes of g_cap bytes */
static size_t g_cap = 0;

static void fail(const char* what) {
  fprintf(stderr, "rank %d: %s\n", g_rank, what);
  fflush(stderr);
  _exit(5);
}

static void sync_all(void) {
  if (g_size > 1) pthread_barrier_wait(&g_sh->barrier);
}

static size_t type_size(int t) {
  if (t == T_DOUBLE) return 8;
  if (t == T_INTEGER) return 4;
  fail("unsupported MPI datatype");
  return 0;
}

void ref_stop(const char* msg, int line) {
  fprintf(stderr, "rank %d: STOP at line %d: %s\n", g_rank, line, msg);
  fflush(stderr);
  _exit(3);
}

void ref_dump(const char* name, const void* data, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%d.bin", g_outdir, name, g_rank);
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(data, 1, bytes, f) != bytes) fail("cannot write a dump file");
  fclose(f);
}

/* wall time of the loop the translator marked (the time loop), written as
   loop_seconds.<rank>.bin when the loop ends */
static struct timespec g_loop_t0;
void ref_timer(int end) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  if (!end) {
    g_loop_t0 = t;
    return;
  }
  const double s = (double)(t.tv_sec - g_loop_t0.tv_sec) + 1e-9 * (double)(t.tv_nsec - g_loop_t0.tv_nsec);
  ref_dump("loop_seconds", &s, sizeof s);
}

void ref_mpi_init(void* ierr) { *(int*)ierr = 0; }
void ref_mpi_finalize(void* ierr) {
  sync_all();
  *(int*)ierr = 0;
}
void ref_mpi_comm_size(void* comm, void* size, void* ierr) {
  (void)comm;
  *(int*)size = g_size;
  *(int*)ierr = 0;
}
void ref_mpi_comm_rank(void* comm, void* rank, void* ierr) {
  (void)comm;
  *(int*)rank = g_rank;
  *(int*)ierr = 0;
}
void ref_mpi_barrier(void* comm, void* ierr) {
  (void)comm;
  sync_all();
  *(int*)ierr = 0;
}

void ref_mpi_sendrecv(void* sbuf, void* scount, void* stype, void* dest, void* stag, void* rbuf,
                      void* rcount, void* rtype, void* source, void* rtag, void* comm,
                      void* status, void* ierr) {
  (void)stag, (void)rtag, (void)comm, (void)status;
  const int d = *(int*)dest, s = *(int*)source;
  const size_t sb = type_size(*(int*)stype) * (size_t)*(int*)scount;
  const size_t rb = type_size(*(int*)rtype) * (size_t)*(int*)rcount;
  if (sb > g_cap || rb > g_cap) fail("message larger than the mailbox");
  if ((d != PROC_NULL && (d < 0 || d >= g_size)) || (s != PROC_NULL && (s < 0 || s >= g_size)))
    fail("rank out of range");
  sync_all();
  if (d != PROC_NULL) {
    memcpy(g_box + (size_t)d * g_cap, sbuf, sb);
    g_sh->from[d] = g_rank;
    g_sh->bytes[d] = (long)sb;
  }
  sync_all();
  if (s != PROC_NULL) {
    if (g_sh->from[g_rank] != s || g_sh->bytes[g_rank] != (long)rb)
      fail("MPI_SENDRECV: no matching message from the named source");
    memcpy(rbuf, g_box + (size_t)g_rank * g_cap, rb);
  }
  g_sh->from[g_rank] = -1;
  sync_all();
  *(int*)ierr = 0;
}

static void reduce_into(void* sbuf, void* rbuf, int n, int type, int op, int to_all, int root) {
  if (n > MAX_REDUCE) fail("reduction longer than the stand-in supports");
  const size_t es = type_size(type);
  sync_all();
  memcpy(g_sh->reduce[g_rank], sbuf, es * (size_t)n);
  sync_all();
  if (to_all || g_rank == root) {
    for (int e = 0; e < n; ++e) {
      if (type == T_DOUBLE) {
        double acc = ((double*)g_sh->reduce[0])[e];
        for (int r = 1; r < g_size; ++r) {
          const double v = ((double*)g_sh->reduce[r])[e];
          acc = op == OP_SUM ? acc + v : op == OP_MAX ? (v > acc ? v : acc) : (v < acc ? v : acc);
        }
        ((double*)rbuf)[e] = acc;
      } else {
        int acc = ((int*)g_sh->reduce[0])[e];
        for (int r = 1; r < g_size; ++r) {
          const int v = ((int*)g_sh->reduce[r])[e];
          acc = op == OP_SUM ? acc + v : op == OP_MAX ? (v > acc ? v : acc) : (v < acc ? v : acc);
        }
        ((int*)rbuf)[e] = acc;
      }
    }
  }
  sync_all();
}

void ref_mpi_reduce(void* sbuf, void* rbuf, void* count, void* type, void* op, void* root,
                    void* comm, void* ierr) {
  (void)comm;
  const int o = *(int*)op;
  if (o != OP_SUM && o != OP_MAX && o != OP_MIN) fail("unsupported reduction");
  reduce_into(sbuf, rbuf, *(int*)count, *(int*)type, o, 0, *(int*)root);
  *(int*)ierr = 0;
}

void ref_mpi_allreduce(void* sbuf, void* rbuf, void* count, void* type, void* op, void* comm,
                       void* ierr) {
  (void)comm;
  const int o = *(int*)op;
  if (o != OP_SUM && o != OP_MAX && o != OP_MIN) fail("unsupported reduction");
  reduce_into(sbuf, rbuf, *(int*)count, *(int*)type, o, 1, 0);
  *(int*)ierr = 0;
}

int main(int argc, char** argv) {
  int np = 1, limit = 900;
  for (int a = 1; a + 1 < argc; a += 2) {
    if (!strcmp(argv[a], "-np")) np = atoi(argv[a + 1]);
    else if (!strcmp(argv[a], "-o")) g_outdir = argv[a + 1];
    else if (!strcmp(argv[a], "-t")) limit = atoi(argv[a + 1]);
    else {
      fprintf(stderr, "usage: %s [-np N] [-o outdir] [-t seconds]\n", argv[0]);
      return 2;
    }
  }
  if (np < 1 || np > MAX_PROCS) {
    fprintf(stderr, "-np must be in [1, %d]\n", MAX_PROCS);
    return 2;
  }
  g_size = np;
  g_cap = (size_t)ref_message_capacity * 8;
  const size_t bytes = sizeof(shared_t) + (size_t)np * g_cap;
  void* mem = mmap(NULL, bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (mem == MAP_FAILED) {
    perror("mmap");
    return 2;
  }
  g_sh = (shared_t*)mem;
  g_box = (unsigned char*)mem + sizeof(shared_t);
  for (int r = 0; r < MAX_PROCS; ++r) g_sh->from[r] = -1;
  if (np == 1) {
    ref_main();
    return 0;
  }
  pthread_barrierattr_t attr;
  pthread_barrierattr_init(&attr);
  pthread_barrierattr_setpshared(&attr, PTHREAD_PROCESS_SHARED);
  if (pthread_barrier_init(&g_sh->barrier, &attr, (unsigned)np)) {
    fprintf(stderr, "pthread_barrier_init failed\n");
    return 2;
  }
  pid_t pids[MAX_PROCS];
  fflush(stdout);
  fflush(stderr);
  for (int r = 0; r < np; ++r) {
    pid_t p = fork();
    if (p < 0) {
      perror("fork");
      for (int q = 0; q < r; ++q) kill(pids[q], SIGKILL);
      return 2;
    }
    if (p == 0) {
      g_rank = r;
      ref_main();
      fflush(stdout);
      _exit(0);
    }
    pids[r] = p;
  }
  /* wait for every rank, polling so that a failed rank or the time limit
     ends the others instead of leaving them at the barrier */
  int left = np, status = 0, rc = 0;
  const time_t t0 = time(NULL);
  while (left > 0) {
    pid_t p = waitpid(-1, &status, WNOHANG);
    if (p > 0) {
      --left;
      if (!WIFEXITED(status) || WEXITSTATUS(status) != 0) {
        rc = WIFEXITED(status) ? WEXITSTATUS(status) : 6;
        break;
      }
      continue;
    }
    if (p < 0 && errno != EINTR) break;
    if (time(NULL) - t0 > limit) {
      fprintf(stderr, "time limit of %d s reached\n", limit);
      rc = 7;
      break;
    }
    usleep(2000);
  }
  if (rc) {
    for (int r = 0; r < np; ++r) kill(pids[r], SIGKILL);
    while (waitpid(-1, &status, 0) > 0) {
    }
  }
  return rc;
}
