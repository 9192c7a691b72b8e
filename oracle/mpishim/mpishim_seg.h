/* TEST INFRASTRUCTURE: layout of the minimal MPI's shared-memory segment (mpishim.c, mpishim_run.c):
 * the header (rank count, a barrier, one mailbox per rank), then one message ring of arena_bytes per
 * rank. */
#ifndef STS_MPISHIM_SEG_H
#define STS_MPISHIM_SEG_H
#include <pthread.h>
#include <stddef.h>

#define SHIM_MAX_RANKS 256

struct shim_box {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  size_t head, tail; /* byte counters of the ring (positions modulo arena_bytes) */
};

struct shim_bar {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  unsigned count, gen;
};

struct shim_header {
  int nranks;
  size_t arena_bytes;
  struct shim_bar bar;
  struct shim_box box[SHIM_MAX_RANKS];
};

static inline size_t shim_header_bytes(void) { return (sizeof(struct shim_header) + 4095) & ~(size_t)4095; }
static inline size_t shim_arena_offset(int nranks, int r, size_t arena_bytes) {
  (void)nranks;
  return shim_header_bytes() + (size_t)r * arena_bytes;
}

#endif
