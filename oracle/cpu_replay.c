/*
 * ORACLE-side CPU baseline — test/benchmark infrastructure only.
 *
 * Replays the benchmark workloads of gallatin_gb300/csrc/workloads.cuh
 * through glibc malloc/free on host threads: the same per-thread size
 * sequence (xorshift64 seeded by splitmix64(seed + tid), or a class trace),
 * the same fill / verify pattern and the same segment-tier requests. Thread
 * ids are split into contiguous ranges, one per worker. The reference has no
 * CPU implementation of its allocator, so glibc is the host-side baseline.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

static uint64_t xorshift64(uint64_t *s) {
  uint64_t x = *s;
  x ^= x << 13;
  x ^= x >> 7;
  x ^= x << 17;
  *s = x;
  return x;
}

typedef struct {
  uint64_t begin, end, n;
  uint32_t rounds;
  uint64_t seed;
  const uint8_t *classes;
  uint32_t seg_every, block_dim;
  uint64_t seg_lo, seg_hi;
  uint64_t size; /* pairs workload when rounds == 0 */
  uint64_t misses, bad;
} job;

static void *run_mixed(void *arg) {
  job *j = (job *)arg;
  uint64_t misses = 0, bad = 0;
  for (uint64_t tid = j->begin; tid < j->end; ++tid) {
    if (j->seg_every && tid % j->block_dim == 0 && (tid / j->block_dim) % j->seg_every == 0) {
      uint64_t k = (tid / j->block_dim) / j->seg_every;
      uint64_t size = j->seg_lo + splitmix64(j->seed + j->n + k) % (j->seg_hi - j->seg_lo + 1);
      uint64_t *p = (uint64_t *)malloc(size);
      if (p) {
        uint64_t last = size / 8 - 2;
        p[0] = tid;
        p[last] = k;
        if (((volatile uint64_t *)p)[0] != tid || ((volatile uint64_t *)p)[last] != k) bad++;
        free(p);
      }
    }
    uint64_t s = splitmix64(j->seed + tid);
    for (uint32_t r = 0; r < j->rounds; ++r) {
      uint32_t cls = j->classes ? j->classes[(uint64_t)r * j->n + tid] : (uint32_t)(xorshift64(&s) % 9);
      uint64_t size = 16ull << cls;
      uint64_t *p = (uint64_t *)malloc(size);
      if (!p) {
        misses++;
        continue;
      }
      uint64_t v = tid ^ r;
      uint64_t words = size / 8;
      for (uint64_t i = 0; i < words; ++i) p[i] = v;
      volatile uint64_t *vp = p;
      for (uint64_t i = 0; i < words; ++i) {
        if (vp[i] != v) {
          bad++;
          break;
        }
      }
      free(p);
    }
  }
  j->misses = misses;
  j->bad = bad;
  return NULL;
}

static void *run_pairs(void *arg) {
  job *j = (job *)arg;
  uint64_t misses = 0, bad = 0;
  for (uint64_t tid = j->begin; tid < j->end; ++tid) {
    uint64_t *p = (uint64_t *)malloc(j->size);
    if (!p) {
      misses++;
      continue;
    }
    p[0] = tid;
    if (((volatile uint64_t *)p)[0] != tid) bad++;
    free(p);
  }
  j->misses = misses;
  j->bad = bad;
  return NULL;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static double run_jobs(void *(*fn)(void *), job *proto, int workers, uint64_t *misses, uint64_t *bad) {
  if (workers < 1) workers = 1;
  if (workers > 1024) workers = 1024;
  job *jobs = (job *)calloc((size_t)workers, sizeof(job));
  pthread_t *th = (pthread_t *)calloc((size_t)workers, sizeof(pthread_t));
  uint64_t total = proto->end - proto->begin;
  for (int w = 0; w < workers; ++w) {
    jobs[w] = *proto;
    jobs[w].begin = proto->begin + total * (uint64_t)w / (uint64_t)workers;
    jobs[w].end = proto->begin + total * (uint64_t)(w + 1) / (uint64_t)workers;
  }
  double t0 = now_s();
  for (int w = 0; w < workers; ++w) pthread_create(&th[w], NULL, fn, &jobs[w]);
  for (int w = 0; w < workers; ++w) pthread_join(th[w], NULL);
  double t1 = now_s();
  *misses = 0;
  *bad = 0;
  for (int w = 0; w < workers; ++w) {
    *misses += jobs[w].misses;
    *bad += jobs[w].bad;
  }
  free(jobs);
  free(th);
  return t1 - t0;
}

/* Mixed workload over thread ids [tid_begin, tid_end) of an n-thread grid.
 * Returns wall seconds. */
double cpu_replay_mixed(uint64_t n, uint64_t tid_begin, uint64_t tid_end, uint32_t rounds, uint64_t seed,
                        const uint8_t *classes, uint32_t seg_every, uint32_t block_dim, uint64_t seg_lo,
                        uint64_t seg_hi, int workers, uint64_t *misses, uint64_t *bad) {
  job proto;
  memset(&proto, 0, sizeof(proto));
  proto.begin = tid_begin;
  proto.end = tid_end;
  proto.n = n;
  proto.rounds = rounds;
  proto.seed = seed;
  proto.classes = classes;
  proto.seg_every = seg_every;
  proto.block_dim = block_dim ? block_dim : 256;
  proto.seg_lo = seg_lo;
  proto.seg_hi = seg_hi;
  return run_jobs(run_mixed, &proto, workers, misses, bad);
}

double cpu_replay_pairs(uint64_t n, uint64_t size, int workers, uint64_t *misses, uint64_t *bad) {
  job proto;
  memset(&proto, 0, sizeof(proto));
  proto.begin = 0;
  proto.end = n;
  proto.n = n;
  proto.size = size;
  return run_jobs(run_pairs, &proto, workers, misses, bad);
}

/* The class trace the mixed workload draws: classes[r * n + tid]. */
void cpu_mixed_classes(uint64_t n, uint32_t rounds, uint64_t seed, uint8_t *out) {
  for (uint64_t tid = 0; tid < n; ++tid) {
    uint64_t s = splitmix64(seed + tid);
    for (uint32_t r = 0; r < rounds; ++r) out[(uint64_t)r * n + tid] = (uint8_t)(xorshift64(&s) % 9);
  }
}

/* Batched request stream (slot << 32 | size; size 0 = free): the requests of
 * a batch are split over the workers, batches run one after another. */
typedef struct {
  const uint64_t *reqs;
  uint64_t begin, end;
  uint64_t *table;
  uint64_t misses;
} batch_job;

static void *run_batch_part(void *arg) {
  batch_job *j = (batch_job *)arg;
  uint64_t misses = 0;
  for (uint64_t i = j->begin; i < j->end; ++i) {
    const uint64_t r = j->reqs[i];
    const uint32_t slot = (uint32_t)(r >> 32);
    const uint32_t size = (uint32_t)r;
    if (size) {
      void *p = malloc(size);
      if (!p) misses++;
      j->table[slot] = (uint64_t)p;
    } else {
      free((void *)j->table[slot]);
      j->table[slot] = 0;
    }
  }
  j->misses = misses;
  return NULL;
}

double cpu_replay_batches(const uint64_t *reqs, const uint64_t *offsets, uint32_t n_batches, uint64_t *table,
                          int workers, uint64_t *misses) {
  if (workers < 1) workers = 1;
  if (workers > 1024) workers = 1024;
  batch_job *jobs = (batch_job *)calloc((size_t)workers, sizeof(batch_job));
  pthread_t *th = (pthread_t *)calloc((size_t)workers, sizeof(pthread_t));
  *misses = 0;
  double t0 = now_s();
  for (uint32_t b = 0; b < n_batches; ++b) {
    const uint64_t lo = offsets[b], n = offsets[b + 1] - offsets[b];
    for (int w = 0; w < workers; ++w) {
      jobs[w].reqs = reqs;
      jobs[w].table = table;
      jobs[w].begin = lo + n * (uint64_t)w / (uint64_t)workers;
      jobs[w].end = lo + n * (uint64_t)(w + 1) / (uint64_t)workers;
      pthread_create(&th[w], NULL, run_batch_part, &jobs[w]);
    }
    for (int w = 0; w < workers; ++w) {
      pthread_join(th[w], NULL);
      *misses += jobs[w].misses;
    }
  }
  double t1 = now_s();
  free(jobs);
  free(th);
  return t1 - t0;
}
