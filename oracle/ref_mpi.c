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
 * It also holds the runtime of the translated programs: STOP, the dump
 * and load hooks of the tests, the timer of the CPU reference timing, and
 * formatted WRITE/OPEN/CLOSE for translated output subroutines.
 *
 * Usage: <program> [-np N] [-o outdir] [-i indir] [-t seconds]. The parent waits for
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
#include <sys/prctl.h>
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
static const char* g_indir = ".";
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

void ref_dump(const char* name, const void* data, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.%d.bin", g_outdir, name, g_rank);
  FILE* f = fopen(path, "wb");
  if (!f || fwrite(data, 1, bytes, f) != bytes) fail("cannot write a dump file");
  fclose(f);
}

/* STOP: the program's dumps of this moment (a hook the translated program
   registers), stop.<rank>.txt with the message, exit status 3 */
static void (*g_stop_hook)(void) = NULL;
void ref_set_stop_hook(void (*hook)(void)) { g_stop_hook = hook; }

void ref_stop(const char* msg, int line) {
  if (g_stop_hook) g_stop_hook();
  char path[4096];
  snprintf(path, sizeof path, "%s/stop.%d.txt", g_outdir, g_rank);
  FILE* f = fopen(path, "w");
  if (f) {
    fprintf(f, "line %d: %s\n", line, msg);
    fclose(f);
  }
  fprintf(stderr, "rank %d: STOP at line %d: %s\n", g_rank, line, msg);
  fflush(stderr);
  _exit(3);
}

/* variables a test fills before the first statement: <indir>/<name>.bin,
   exactly the variable's size */
void ref_load(const char* name, void* data, size_t bytes) {
  char path[4096];
  snprintf(path, sizeof path, "%s/%s.bin", g_indir, name);
  FILE* f = fopen(path, "rb");
  if (!f || fread(data, 1, bytes, f) != bytes || fgetc(f) != EOF) fail("cannot load an input file");
  fclose(f);
}

/* Formatted output: one record is built, then written to a unit (a line
   of its file) or into a character variable (blank-padded). Iw.m edits
   right-justify in w columns with at least m digits (w asterisks when the
   number does not fit); list-directed integers take 12 columns and strings
   a leading blank, the layout of gfortran's list-directed records. */
static char g_rec[16384];
static size_t g_rec_n;
static FILE* g_units[128];

static void rec_put(const char* s, size_t n) {
  if (g_rec_n + n >= sizeof g_rec) fail("output record too long");
  memcpy(g_rec + g_rec_n, s, n);
  g_rec_n += n;
}
void ref_rec_begin(void) { g_rec_n = 0; }
void ref_put_s(const char* s) { rec_put(s, strlen(s)); }
void ref_put_i(long v, int w, int m) {
  char digits[32], body[64];
  int nd = snprintf(digits, sizeof digits, "%ld", v < 0 ? -v : v);
  if (v == 0 && m == 0) nd = 0;
  const int mm = m < 0 ? 1 : m;
  size_t n = 0;
  if (v < 0) body[n++] = '-';
  for (int k = nd; k < mm && n < 40; ++k) body[n++] = '0';
  memcpy(body + n, digits, (size_t)nd);
  n += (size_t)nd;
  if ((int)n > w) {
    for (int k = 0; k < w; ++k) rec_put("*", 1);
    return;
  }
  for (int k = (int)n; k < w; ++k) rec_put(" ", 1);
  rec_put(body, n);
}
void ref_ld_i(long v) {
  char b[32];
  const int n = snprintf(b, sizeof b, "%12ld", v);
  rec_put(b, (size_t)n);
}
/* list-directed reals: 9 significant digits for single precision, 17 for
   double, so that reading the text back gives the value exactly */
void ref_ld_r(double v, int kind) {
  char b[48];
  const int n = snprintf(b, sizeof b, kind == 1 ? "  %.8E" : "  %.16E", v);
  rec_put(b, (size_t)n);
}
void ref_ld_s(const char* s) {
  rec_put(" ", 1);
  ref_put_s(s);
}
void ref_rec_internal(char* buf, int len) {
  const size_t n = g_rec_n < (size_t)len ? g_rec_n : (size_t)len;
  memcpy(buf, g_rec, n);
  memset(buf + n, ' ', (size_t)len - n);
  buf[len] = 0;
}
void ref_open(int unit, const char* name, int len) {
  char path[4096];
  size_t n = len < 0 ? strlen(name) : (size_t)len;
  while (n > 0 && name[n - 1] == ' ') --n;        /* Fortran names are blank-padded */
  if (unit < 0 || unit >= 128 || n == 0 || n >= sizeof path) fail("bad OPEN");
  memcpy(path, name, n);
  path[n] = 0;
  if (g_units[unit]) fclose(g_units[unit]);
  g_units[unit] = fopen(path, "w");
  if (!g_units[unit]) fail("OPEN failed");
}
void ref_rec_unit(int unit) {
  if (unit < 0 || unit >= 128 || !g_units[unit]) fail("WRITE to a unit that is not open");
  if (fwrite(g_rec, 1, g_rec_n, g_units[unit]) != g_rec_n || fputc('\n', g_units[unit]) == EOF)
    fail("WRITE failed");
}
void ref_close(int unit) {
  if (unit >= 0 && unit < 128 && g_units[unit]) {
    fclose(g_units[unit]);
    g_units[unit] = NULL;
  }
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
    else if (!strcmp(argv[a], "-i")) g_indir = argv[a + 1];
    else if (!strcmp(argv[a], "-t")) limit = atoi(argv[a + 1]);
    else {
      fprintf(stderr, "usage: %s [-np N] [-o outdir] [-i indir] [-t seconds]\n", argv[0]);
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
      /* a rank never outlives the parent: killed from outside, the parent
         cannot end the ranks waiting at the barrier itself */
      prctl(PR_SET_PDEATHSIG, SIGKILL);
      if (getppid() == 1) _exit(8);
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
