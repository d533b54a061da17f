/*
 * mpi_shim.c -- forked-process MPI subset (see mpi.h).  TEST INFRASTRUCTURE.
 *
 * MPI_Init forks SHIM_MPI_NP-1 children; the parent is rank 0.  A shared
 * anonymous mapping holds a sense-reversing barrier and one message slot per
 * rank.  MPI_Reduce copies every contribution into its slot and the root sums
 * slots 0..P-1 in rank order (deterministic); MPI_Bcast copies through the
 * root's slot.  Children die with the parent (PR_SET_PDEATHSIG); the parent
 * notices a child that exits before MPI_Finalize while it waits in a barrier
 * and then aborts every rank, so a failing rank never leaves the others
 * spinning.  Slot size: SHIM_MPI_SLOT_MB (default 512) megabytes.
 */
#define _GNU_SOURCE
#include "mpi.h"

#include <errno.h>
#include <sched.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/prctl.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#define SHIM_MAXP 512

typedef struct {
  volatile int count;
  volatile int sense;
  volatile int abort_flag;
  volatile int finalized[SHIM_MAXP];
} shim_ctl;

static int g_rank = 0, g_size = 1;
static shim_ctl *g_ctl = NULL;
static char *g_slots = NULL;
static size_t g_slot_bytes = 0;
static int g_local_sense = 0;
static pid_t g_child[SHIM_MAXP];
static int g_child_done[SHIM_MAXP];
static int g_live_comms[64];

static void shim_die(const char *msg) {
  fprintf(stderr, "shim MPI (rank %d): %s\n", g_rank, msg);
  fflush(stderr);
  if (g_ctl) __atomic_store_n(&g_ctl->abort_flag, 1, __ATOMIC_SEQ_CST);
  _exit(1);
}

/* Rank 0 only: reap children that already exited; one that exits before
 * finalising (or with a failure status) aborts the run. */
static void check_children(void) {
  if (g_rank != 0) return;
  for (int r = 1; r < g_size; r++) {
    if (g_child_done[r]) continue;
    int st = 0;
    pid_t p = waitpid(g_child[r], &st, WNOHANG);
    if (p == g_child[r]) {
      g_child_done[r] = 1;
      int ok = WIFEXITED(st) && WEXITSTATUS(st) == 0 && g_ctl->finalized[r];
      if (!ok) shim_die("a rank exited before MPI_Finalize");
    }
  }
}

static void shim_barrier(void) {
  if (g_size == 1) return;
  g_local_sense = !g_local_sense;
  int arrived = __atomic_add_fetch(&g_ctl->count, 1, __ATOMIC_ACQ_REL);
  if (arrived == g_size) {
    __atomic_store_n(&g_ctl->count, 0, __ATOMIC_RELAXED);
    __atomic_store_n(&g_ctl->sense, g_local_sense, __ATOMIC_RELEASE);
    return;
  }
  long spins = 0;
  while (__atomic_load_n(&g_ctl->sense, __ATOMIC_ACQUIRE) != g_local_sense) {
    if (__atomic_load_n(&g_ctl->abort_flag, __ATOMIC_ACQUIRE))
      shim_die("aborting because another rank failed");
    if (++spins > 2000) {
      struct timespec ts = {0, 20000};
      nanosleep(&ts, NULL);
      if ((spins & 255) == 0) check_children();
    } else if ((spins & 63) == 0) {
      sched_yield();
    }
  }
}

static size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_LONG: return sizeof(long);
    case MPI_DOUBLE: return sizeof(double);
    default: shim_die("unsupported datatype");
  }
  return 0;
}

static void check_comm(MPI_Comm comm) {
  if (comm == MPI_COMM_WORLD) return;
  if (comm > 0 && comm < 64 && g_live_comms[comm]) return;
  shim_die("unsupported communicator");
}

int MPI_Init(int *argc, char ***argv) {
  (void)argc;
  (void)argv;
  const char *np = getenv("SHIM_MPI_NP");
  g_size = np ? atoi(np) : 2;
  if (g_size < 1 || g_size > SHIM_MAXP) shim_die("bad SHIM_MPI_NP");
  const char *mb = getenv("SHIM_MPI_SLOT_MB");
  g_slot_bytes = (size_t)(mb ? atol(mb) : 512) << 20;
  size_t ctl_bytes = (sizeof(shim_ctl) + 4095) & ~(size_t)4095;
  void *base = mmap(NULL, ctl_bytes + g_slot_bytes * (size_t)g_size,
                    PROT_READ | PROT_WRITE,
                    MAP_SHARED | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
  if (base == MAP_FAILED) shim_die("mmap of the shared area failed");
  g_ctl = (shim_ctl *)base;
  memset((void *)g_ctl, 0, sizeof(shim_ctl));
  g_slots = (char *)base + ctl_bytes;
  fflush(stdout);
  fflush(stderr);
  pid_t parent = getpid();
  for (int r = 1; r < g_size; r++) {
    pid_t p = fork();
    if (p < 0) shim_die("fork failed");
    if (p == 0) {
      prctl(PR_SET_PDEATHSIG, SIGKILL);
      if (getppid() != parent) _exit(1);
      g_rank = r;
      return MPI_SUCCESS;
    }
    g_child[r] = p;
  }
  g_rank = 0;
  return MPI_SUCCESS;
}

int MPI_Finalize(void) {
  shim_barrier();
  __atomic_store_n(&g_ctl->finalized[g_rank], 1, __ATOMIC_SEQ_CST);
  fflush(stdout);
  fflush(stderr);
  if (g_rank == 0) {
    int failed = 0;
    for (int r = 1; r < g_size; r++) {
      if (g_child_done[r]) continue;
      int st = 0;
      while (waitpid(g_child[r], &st, 0) < 0 && errno == EINTR) {
      }
      if (!(WIFEXITED(st) && WEXITSTATUS(st) == 0)) failed = 1;
    }
    if (failed) shim_die("a rank failed after MPI_Finalize");
  }
  return MPI_SUCCESS;
}

int MPI_Abort(MPI_Comm comm, int errorcode) {
  (void)comm;
  if (g_ctl) __atomic_store_n(&g_ctl->abort_flag, 1, __ATOMIC_SEQ_CST);
  _exit(errorcode ? errorcode : 1);
}

int MPI_Comm_size(MPI_Comm comm, int *size) {
  check_comm(comm);
  *size = g_size;
  return MPI_SUCCESS;
}

int MPI_Comm_rank(MPI_Comm comm, int *rank) {
  check_comm(comm);
  *rank = g_rank;
  return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm) {
  check_comm(comm);
  shim_barrier();
  return MPI_SUCCESS;
}

int MPI_Reduce(const void *sendbuf, void *recvbuf, int count,
               MPI_Datatype datatype, MPI_Op op, int root, MPI_Comm comm) {
  check_comm(comm);
  if (op != MPI_SUM) shim_die("only MPI_SUM is supported");
  size_t es = type_size(datatype), bytes = es * (size_t)count;
  if (bytes > g_slot_bytes) shim_die("message larger than SHIM_MPI_SLOT_MB");
  memcpy(g_slots + g_slot_bytes * (size_t)g_rank, sendbuf, bytes);
  shim_barrier();
  if (g_rank == root) {
    for (int i = 0; i < count; i++) {
      if (datatype == MPI_DOUBLE) {
        double acc = ((const double *)g_slots)[i];
        for (int r = 1; r < g_size; r++)
          acc += ((const double *)(g_slots + g_slot_bytes * (size_t)r))[i];
        ((double *)recvbuf)[i] = acc;
      } else if (datatype == MPI_LONG) {
        long acc = ((const long *)g_slots)[i];
        for (int r = 1; r < g_size; r++)
          acc += ((const long *)(g_slots + g_slot_bytes * (size_t)r))[i];
        ((long *)recvbuf)[i] = acc;
      } else {
        int acc = ((const int *)g_slots)[i];
        for (int r = 1; r < g_size; r++)
          acc += ((const int *)(g_slots + g_slot_bytes * (size_t)r))[i];
        ((int *)recvbuf)[i] = acc;
      }
    }
  }
  shim_barrier();
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count,
                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm) {
  MPI_Reduce(sendbuf, recvbuf, count, datatype, op, 0, comm);
  return MPI_Bcast(recvbuf, count, datatype, 0, comm);
}

int MPI_Bcast(void *buffer, int count, MPI_Datatype datatype, int root,
              MPI_Comm comm) {
  check_comm(comm);
  size_t bytes = type_size(datatype) * (size_t)count;
  if (bytes > g_slot_bytes) shim_die("message larger than SHIM_MPI_SLOT_MB");
  char *slot = g_slots + g_slot_bytes * (size_t)root;
  if (g_rank == root) memcpy(slot, buffer, bytes);
  shim_barrier();
  if (g_rank != root) memcpy(buffer, slot, bytes);
  shim_barrier();
  return MPI_SUCCESS;
}

/* Groups are process-local rank lists. */
static int *g_groups[64];
static int g_group_n[64];

int MPI_Comm_group(MPI_Comm comm, MPI_Group *group) {
  check_comm(comm);
  for (int g = 0; g < 64; g++)
    if (!g_groups[g]) {
      g_groups[g] = (int *)malloc(sizeof(int) * g_size);
      for (int r = 0; r < g_size; r++) g_groups[g][r] = r;
      g_group_n[g] = g_size;
      *group = g;
      return MPI_SUCCESS;
    }
  shim_die("too many groups");
  return 1;
}

int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3],
                         MPI_Group *newgroup) {
  if (group < 0 || group >= 64 || !g_groups[group]) shim_die("bad group");
  int tmp[SHIM_MAXP], cnt = 0;
  for (int i = 0; i < n; i++) {
    int a = ranges[i][0], b = ranges[i][1], s = ranges[i][2];
    if (s == 0) shim_die("zero stride in MPI_Group_range_incl");
    for (int r = a; s > 0 ? r <= b : r >= b; r += s) {
      if (r < 0 || r >= g_group_n[group] || cnt >= SHIM_MAXP)
        shim_die("bad range in MPI_Group_range_incl");
      tmp[cnt++] = g_groups[group][r];
    }
  }
  for (int g = 0; g < 64; g++)
    if (!g_groups[g]) {
      g_groups[g] = (int *)malloc(sizeof(int) * (cnt ? cnt : 1));
      memcpy(g_groups[g], tmp, sizeof(int) * cnt);
      g_group_n[g] = cnt;
      *newgroup = g;
      return MPI_SUCCESS;
    }
  shim_die("too many groups");
  return 1;
}

int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm *newcomm) {
  check_comm(comm);
  if (group < 0 || group >= 64 || !g_groups[group]) shim_die("bad group");
  int full = g_group_n[group] == g_size;
  for (int r = 0; full && r < g_size; r++) full = g_groups[group][r] == r;
  if (!full) shim_die("only communicators over every rank are supported");
  for (int c = 1; c < 64; c++)
    if (!g_live_comms[c]) {
      g_live_comms[c] = 1;
      *newcomm = c;
      return MPI_SUCCESS;
    }
  shim_die("too many communicators");
  return 1;
}

int MPI_Comm_free(MPI_Comm *comm) {
  if (*comm > 0 && *comm < 64) g_live_comms[*comm] = 0;
  *comm = MPI_COMM_NULL;
  return MPI_SUCCESS;
}

int MPI_Group_free(MPI_Group *group) {
  if (*group >= 0 && *group < 64 && g_groups[*group]) {
    free(g_groups[*group]);
    g_groups[*group] = NULL;
  }
  *group = MPI_GROUP_NULL;
  return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype datatype, int dest,
             int tag, MPI_Comm comm) {
  (void)buf; (void)count; (void)datatype; (void)dest; (void)tag; (void)comm;
  shim_die("MPI_Send is only used by the reference when nsubm > 1");
  return 1;
}

int MPI_Recv(void *buf, int count, MPI_Datatype datatype, int source, int tag,
             MPI_Comm comm, MPI_Status *status) {
  (void)buf; (void)count; (void)datatype; (void)source; (void)tag;
  (void)comm; (void)status;
  shim_die("MPI_Recv is only used by the reference when nsubm > 1");
  return 1;
}
