/*
 * TEST INFRASTRUCTURE: launcher of the minimal MPI (mpishim.c).
 *
 *   mpishim_run N program [args...]
 *
 * creates the shared segment (one message ring of 256 MB per rank, sparse: only used pages take
 * memory), starts N processes of `program` in the current directory with MPISHIM_SHM,
 * MPISHIM_RANK and MPISHIM_SIZE set, waits for all of them and removes the segment.  Exit status:
 * the first non-zero one of the ranks, else 0.
 */
#define _GNU_SOURCE
#include <fcntl.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <sys/wait.h>
#include <unistd.h>

#include "mpishim_seg.h"

static void shared_mutex(pthread_mutex_t* m, pthread_cond_t* c) {
  pthread_mutexattr_t ma;
  pthread_condattr_t ca;
  pthread_mutexattr_init(&ma);
  pthread_mutexattr_setpshared(&ma, PTHREAD_PROCESS_SHARED);
  pthread_mutex_init(m, &ma);
  pthread_condattr_init(&ca);
  pthread_condattr_setpshared(&ca, PTHREAD_PROCESS_SHARED);
  pthread_cond_init(c, &ca);
}

int main(int argc, char** argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: mpishim_run N program [args...]\n");
    return 2;
  }
  const int n = atoi(argv[1]);
  if (n < 1 || n > SHIM_MAX_RANKS) {
    fprintf(stderr, "mpishim_run: N must be 1..%d\n", SHIM_MAX_RANKS);
    return 2;
  }
  const size_t arena = (size_t)256 << 20;
  const size_t bytes = shim_header_bytes() + (size_t)n * arena;
  char name[64];
  snprintf(name, sizeof name, "/mpishim_%d", (int)getpid());
  const int fd = shm_open(name, O_CREAT | O_EXCL | O_RDWR, 0600);
  if (fd < 0 || ftruncate(fd, (off_t)bytes) != 0) {
    perror("mpishim_run: shared segment");
    return 2;
  }
  struct shim_header* h = (struct shim_header*)mmap(NULL, shim_header_bytes(), PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
  close(fd);
  if (h == MAP_FAILED) {
    perror("mpishim_run: mmap");
    shm_unlink(name);
    return 2;
  }
  memset(h, 0, sizeof *h);
  h->nranks = n;
  h->arena_bytes = arena;
  shared_mutex(&h->bar.mu, &h->bar.cv);
  for (int r = 0; r < n; r++) shared_mutex(&h->box[r].mu, &h->box[r].cv);
  munmap(h, shim_header_bytes());
  pid_t* pids = (pid_t*)calloc((size_t)n, sizeof(pid_t));
  for (int r = 0; r < n; r++) {
    const pid_t p = fork();
    if (p == 0) {
      char rank[16], size[16];
      snprintf(rank, sizeof rank, "%d", r);
      snprintf(size, sizeof size, "%d", n);
      setenv("MPISHIM_SHM", name, 1);
      setenv("MPISHIM_RANK", rank, 1);
      setenv("MPISHIM_SIZE", size, 1);
      execvp(argv[2], argv + 2);
      perror("mpishim_run: exec");
      _exit(127);
    }
    pids[r] = p;
  }
  int rc = 0;
  for (int r = 0; r < n; r++) {
    int st = 0;
    waitpid(pids[r], &st, 0);
    const int code = WIFEXITED(st) ? WEXITSTATUS(st) : 128 + WTERMSIG(st);
    if (code && !rc) rc = code;
  }
  shm_unlink(name);
  free(pids);
  return rc;
}
