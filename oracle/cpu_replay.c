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
  int zeroed;    /* mixed: calloc, and check every byte reads zero first */
  uint64_t *table; /* fill/drain: one pointer per thread id */
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
      uint64_t *p = (uint64_t *)(j->zeroed ? calloc(1, size) : malloc(size));
      if (!p) {
        misses++;
        continue;
      }
      uint64_t v = tid ^ r;
      uint64_t words = size / 8;
      if (j->zeroed) {
        uint64_t seen = 0;
        for (uint64_t i = 0; i < words; ++i) seen |= ((volatile uint64_t *)p)[i];
        if (seen) bad++;
      }
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

/* the fused fill/drain workload of gallatin_gb300/csrc/spill_workloads.cuh:
 * thread i's size is 16 << classes[i]; fill writes i and ~i to the first and
 * last u64, drain checks them and frees */
static void *run_fill(void *arg) {
  job *j = (job *)arg;
  uint64_t misses = 0;
  for (uint64_t i = j->begin; i < j->end; ++i) {
    uint64_t size = 16ull << j->classes[i];
    uint64_t *p = (uint64_t *)malloc(size);
    j->table[i] = (uint64_t)p;
    if (!p) {
      misses++;
      continue;
    }
    p[0] = i;
    p[size / 8 - 1] = ~i;
  }
  j->misses = misses;
  return NULL;
}

static void *run_drain(void *arg) {
  job *j = (job *)arg;
  uint64_t bad = 0;
  for (uint64_t i = j->begin; i < j->end; ++i) {
    uint64_t *p = (uint64_t *)j->table[i];
    if (!p) continue;
    uint64_t size = 16ull << j->classes[i];
    if (((volatile uint64_t *)p)[0] != i || ((volatile uint64_t *)p)[size / 8 - 1] != ~i) bad++;
    free(p);
    j->table[i] = 0;
  }
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

/* The mixed workload through calloc: every allocation is checked to read
 * zero before the fill (bad counts those that did not). */
double cpu_replay_mixed_zeroed(uint64_t n, uint64_t tid_begin, uint64_t tid_end, uint32_t rounds, uint64_t seed,
                               const uint8_t *classes, int workers, uint64_t *misses, uint64_t *bad) {
  job proto;
  memset(&proto, 0, sizeof(proto));
  proto.begin = tid_begin;
  proto.end = tid_end;
  proto.n = n;
  proto.rounds = rounds;
  proto.seed = seed;
  proto.classes = classes;
  proto.block_dim = 256;
  proto.zeroed = 1;
  return run_jobs(run_mixed, &proto, workers, misses, bad);
}

/* Fill then drain n allocations (table: n u64 the caller provides); returns
 * the wall seconds of both phases. */
double cpu_replay_fill_drain(uint64_t n, const uint8_t *classes, uint64_t *table, int workers, uint64_t *misses,
                             uint64_t *bad) {
  job proto;
  memset(&proto, 0, sizeof(proto));
  proto.begin = 0;
  proto.end = n;
  proto.n = n;
  proto.classes = classes;
  proto.table = table;
  uint64_t m = 0, b = 0, m2 = 0, b2 = 0;
  double secs = run_jobs(run_fill, &proto, workers, &m, &b);
  secs += run_jobs(run_drain, &proto, workers, &m2, &b2);
  *misses = m;
  *bad = b2;
  return secs;
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

/* ---- serving ------------------------------------------------------------
 * Token `pos` of stream `id` and the checksum a finished stream reports
 * (gallatin_gb300/csrc/serving.cuh): sum of token * (2 * pos + 1) mod 2^64. */
static uint64_t serve_token(uint64_t seed, uint32_t id, uint32_t pos) {
  return splitmix64(seed ^ (((uint64_t)id << 16) | pos));
}

typedef struct {
  uint64_t begin, end, seed;
  const uint32_t *tokens;
  uint64_t *out;
} sum_job;

static void *run_sums(void *arg) {
  sum_job *j = (sum_job *)arg;
  for (uint64_t i = j->begin; i < j->end; ++i) {
    uint64_t acc = 0;
    for (uint32_t p = 0; p < j->tokens[i]; ++p) acc += serve_token(j->seed, (uint32_t)i, p) * (2ull * p + 1);
    j->out[i] = acc;
  }
  return NULL;
}

void cpu_serving_checksums(uint64_t n, const uint32_t *tokens, uint64_t seed, uint64_t *out, int workers) {
  if (workers < 1) workers = 1;
  if (workers > 256) workers = 256;
  sum_job jobs[256];
  pthread_t th[256];
  for (int w = 0; w < workers; ++w) {
    jobs[w].begin = n * (uint64_t)w / (uint64_t)workers;
    jobs[w].end = n * (uint64_t)(w + 1) / (uint64_t)workers;
    jobs[w].seed = seed;
    jobs[w].tokens = tokens;
    jobs[w].out = out;
    pthread_create(&th[w], NULL, run_sums, &jobs[w]);
  }
  for (int w = 0; w < workers; ++w) pthread_join(th[w], NULL);
}

/* Latency bucket of the serving histogram: ns < 32 exact, then 32 linear
 * buckets per octave (864 buckets). */
static uint32_t serve_bucket(uint64_t ns) {
  if (ns < 32) return (uint32_t)ns;
  int e = 63 - __builtin_clzll(ns);
  if (e > 30) return 863;
  return 32u + (uint32_t)(e - 5) * 32u + ((uint32_t)(ns >> (e - 5)) & 31u);
}

typedef struct serve_shared serve_shared;
typedef struct {
  serve_shared *sh;
  int w;
  uint64_t hist[864];
} serve_worker;

struct serve_shared {
  uint32_t steps, tokens_per_page, workers;
  uint64_t page_bytes, seed, n;
  const uint32_t *tokens, *pages;
  const uint64_t *step_begin; /* streams admitted at step s: [step_begin[s], step_begin[s+1]) */
  uint64_t *checksum;
  void ***table;  /* per stream: its pages */
  uint32_t *held; /* per stream */
  uint32_t *active;
  uint64_t n_active;
  uint8_t *done;
  uint64_t nulls;
  pthread_barrier_t bar;
};

static void *serve_run(void *arg) {
  serve_worker *wk = (serve_worker *)arg;
  serve_shared *sh = wk->sh;
  uint64_t nulls = 0;
  for (uint32_t s = 0; s < sh->steps; ++s) {
    if (wk->w == 0) {
      /* compact survivors, then append this step's admissions */
      uint64_t m = 0;
      for (uint64_t i = 0; i < sh->n_active; ++i)
        if (!sh->done[sh->active[i]]) sh->active[m++] = sh->active[i];
      for (uint64_t id = sh->step_begin[s]; id < sh->step_begin[s + 1]; ++id) {
        sh->table[id] = (void **)malloc(sizeof(void *) * sh->pages[id]);
        sh->held[id] = 0;
        sh->active[m++] = (uint32_t)id;
      }
      sh->n_active = m;
    }
    pthread_barrier_wait(&sh->bar);
    const uint64_t lo = sh->n_active * (uint64_t)wk->w / sh->workers;
    const uint64_t hi = sh->n_active * (uint64_t)(wk->w + 1) / sh->workers;
    for (uint64_t i = lo; i < hi; ++i) {
      const uint32_t id = sh->active[i];
      struct timespec t0, t1;
      clock_gettime(CLOCK_MONOTONIC, &t0);
      uint64_t *p = (uint64_t *)malloc(sh->page_bytes);
      clock_gettime(CLOCK_MONOTONIC, &t1);
      wk->hist[serve_bucket((uint64_t)(t1.tv_sec - t0.tv_sec) * 1000000000ull + (uint64_t)(t1.tv_nsec - t0.tv_nsec))]++;
      if (!p) {
        nulls++;
        continue;
      }
      const uint32_t j = sh->held[id];
      const uint32_t base = j * sh->tokens_per_page;
      const uint32_t len = sh->tokens[id];
      const uint32_t cnt = len - base < sh->tokens_per_page ? len - base : sh->tokens_per_page;
      for (uint32_t t = 0; t < cnt; ++t) p[t] = serve_token(sh->seed, id, base + t);
      sh->table[id][j] = p;
      sh->held[id] = j + 1;
      if (j + 1 == sh->pages[id]) {
        uint64_t acc = 0;
        for (uint32_t q = 0; q <= j; ++q) {
          const uint64_t *pg = (const uint64_t *)sh->table[id][q];
          const uint32_t b = q * sh->tokens_per_page;
          const uint32_t c = len - b < sh->tokens_per_page ? len - b : sh->tokens_per_page;
          for (uint32_t t = 0; t < c; ++t) acc += pg[t] * (2ull * (b + t) + 1);
          free((void *)pg);
        }
        sh->checksum[id] = acc;
        free(sh->table[id]);
        sh->table[id] = NULL;
        sh->done[id] = 1;
      }
    }
    pthread_barrier_wait(&sh->bar);
  }
  __atomic_fetch_add(&sh->nulls, nulls, __ATOMIC_RELAXED);
  return NULL;
}

/* glibc malloc/free through the serving schedule: admit_step[i] (from the
 * admission model) says when stream i starts; a worker per contiguous share
 * of the active streams takes each stream's page per step, a barrier closes
 * the step. Unfinished streams are freed after the last step (untimed).
 * Returns wall seconds of the steps; hist gets the per-malloc latency. */
double cpu_replay_serving(uint64_t n, const uint32_t *tokens, const uint32_t *pages, const uint32_t *admit_step,
                          uint32_t steps, uint32_t tokens_per_page, uint64_t page_bytes, uint64_t seed, int workers,
                          uint64_t *checksum, uint64_t *hist, uint64_t *nulls) {
  if (workers < 1) workers = 1;
  if (workers > 256) workers = 256;
  serve_shared sh;
  memset(&sh, 0, sizeof(sh));
  sh.steps = steps;
  sh.tokens_per_page = tokens_per_page;
  sh.workers = (uint32_t)workers;
  sh.page_bytes = page_bytes;
  sh.seed = seed;
  sh.n = n;
  sh.tokens = tokens;
  sh.pages = pages;
  sh.checksum = checksum;
  uint64_t *step_begin = (uint64_t *)calloc(steps + 1, sizeof(uint64_t));
  /* admissions are first come first served: stream ids admitted at step s
   * form one run, after those of earlier steps */
  uint64_t id = 0;
  for (uint32_t s = 0; s < steps; ++s) {
    step_begin[s] = id;
    while (id < n && admit_step[id] == s) ++id;
  }
  step_begin[steps] = id;
  sh.step_begin = step_begin;
  sh.table = (void ***)calloc(n ? n : 1, sizeof(void **));
  sh.held = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  sh.active = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
  sh.done = (uint8_t *)calloc(n ? n : 1, 1);
  for (uint64_t i = 0; i < n; ++i) checksum[i] = 0;
  pthread_barrier_init(&sh.bar, NULL, (unsigned)workers);
  serve_worker *wk = (serve_worker *)calloc((size_t)workers, sizeof(serve_worker));
  pthread_t *th = (pthread_t *)calloc((size_t)workers, sizeof(pthread_t));
  const double t0 = now_s();
  for (int w = 0; w < workers; ++w) {
    wk[w].sh = &sh;
    wk[w].w = w;
    pthread_create(&th[w], NULL, serve_run, &wk[w]);
  }
  for (int w = 0; w < workers; ++w) pthread_join(th[w], NULL);
  const double t1 = now_s();
  for (int b = 0; b < 864; ++b) {
    hist[b] = 0;
    for (int w = 0; w < workers; ++w) hist[b] += wk[w].hist[b];
  }
  for (uint64_t i = 0; i < n; ++i) {
    if (sh.table[i]) {
      for (uint32_t q = 0; q < sh.held[i]; ++q) free(sh.table[i][q]);
      free(sh.table[i]);
    }
  }
  *nulls = sh.nulls;
  pthread_barrier_destroy(&sh.bar);
  free(step_begin);
  free(sh.table);
  free(sh.held);
  free(sh.active);
  free(sh.done);
  free(wk);
  free(th);
  return t1 - t0;
}

/* ---- allocator-backed data structures -------------------------------------
 * The chained hash table and the doubling vectors of
 * gallatin_gb300/structures.cuh with glibc malloc/free for nodes and
 * backings, on host threads: same node shape (next, 7 keys, 7 values), same
 * bucket (MurmurHash64A of the key mod nbuckets, as the reference table does,
 * chaining_table.cuh:235), same keys (splitmix64(seed + i)), values
 * (splitmix64(key)) and erased half, same vector items and doubling. */
static uint64_t ds_murmur(uint64_t key, uint64_t seed) {
  /* MurmurHash64A of one 8-byte key (reference hashers/murmurhash.cuh:20-61) */
  const uint64_t m = 0xc6a4a7935bd1e995ull;
  const int r = 47;
  uint64_t h = seed ^ (8 * m);
  uint64_t k = key;
  k *= m;
  k ^= k >> r;
  k *= m;
  h ^= k;
  h *= m;
  h ^= h >> r;
  h *= m;
  h ^= h >> r;
  return h;
}

#define DS_EMPTY (~0ull)
typedef struct ds_node {
  struct ds_node *next;
  uint64_t keys[7];
  uint64_t vals[7];
} ds_node;

typedef struct {
  ds_node **heads;
  uint64_t nbuckets, tseed, kseed, begin, end;
  int op; /* 0 insert, 1 erase half, 2 reinsert half, 3 query all, 4 compact, 5 clear */
  uint64_t bad;
} ds_job;

static int ds_half(uint64_t seed, uint64_t i) { return (int)(splitmix64(seed ^ (i * 0x9E3779B97F4A7C15ull)) & 1); }

static int ds_insert(ds_job *j, uint64_t key, uint64_t val) {
  ds_node **link = j->heads + ds_murmur(key, j->tseed) % j->nbuckets;
  ds_node *b = __atomic_load_n(link, __ATOMIC_ACQUIRE);
  for (int hop = 0; hop < (1 << 16); ++hop) {
    if (!b) {
      ds_node *nb = (ds_node *)malloc(sizeof(ds_node));
      if (!nb) return 0;
      nb->next = NULL;
      for (int i = 0; i < 7; ++i) nb->keys[i] = DS_EMPTY;
      ds_node *expect = NULL;
      if (__atomic_compare_exchange_n(link, &expect, nb, 0, __ATOMIC_ACQ_REL, __ATOMIC_ACQUIRE)) {
        b = nb;
      } else {
        free(nb);
        b = expect;
      }
    }
    for (int i = 0; i < 7; ++i) {
      uint64_t e = DS_EMPTY;
      if (__atomic_load_n(&b->keys[i], __ATOMIC_RELAXED) == DS_EMPTY &&
          __atomic_compare_exchange_n(&b->keys[i], &e, key, 0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED)) {
        b->vals[i] = val;
        return 1;
      }
    }
    link = &b->next;
    b = __atomic_load_n(link, __ATOMIC_ACQUIRE);
  }
  return 0;
}

static void *ds_run(void *arg) {
  ds_job *j = (ds_job *)arg;
  uint64_t bad = 0;
  for (uint64_t i = j->begin; i < j->end; ++i) {
    if (j->op == 4 || j->op == 5) {
      ds_node **link = j->heads + i;
      while (*link) {
        ds_node *b = *link;
        int empty = 1;
        for (int q = 0; q < 7; ++q) empty &= b->keys[q] == DS_EMPTY;
        if (j->op == 5 || empty) {
          *link = b->next;
          free(b);
        } else {
          link = &b->next;
        }
      }
      continue;
    }
    const uint64_t key = splitmix64(j->kseed + i);
    const int half = ds_half(j->kseed, i);
    if (j->op == 0 || (j->op == 2 && half)) {
      bad += !ds_insert(j, key, splitmix64(key));
    } else if (j->op == 1 && half) {
      int found = 0;
      for (ds_node *b = j->heads[ds_murmur(key, j->tseed) % j->nbuckets]; b && !found; b = b->next)
        for (int q = 0; q < 7 && !found; ++q) {
          uint64_t e = key;
          if (b->keys[q] == key &&
              __atomic_compare_exchange_n(&b->keys[q], &e, DS_EMPTY, 0, __ATOMIC_ACQ_REL, __ATOMIC_RELAXED))
            found = 1;
        }
      bad += !found;
    } else if (j->op == 3) {
      int found = 0;
      for (ds_node *b = j->heads[ds_murmur(key, j->tseed) % j->nbuckets]; b && !found; b = b->next)
        for (int q = 0; q < 7 && !found; ++q)
          if (b->keys[q] == key) found = b->vals[q] == splitmix64(key) ? 1 : 2;
      bad += found != 1;
    }
  }
  j->bad = bad;
  return NULL;
}

/* Insert n keys, erase half, compact, reinsert the half (timed), then check
 * every key (untimed) and free every node. Returns the timed seconds; *bad
 * counts failed inserts, missing erases and wrong or missing keys. */
double cpu_table(uint64_t n, uint64_t nbuckets, uint64_t tseed, uint64_t kseed, int workers, uint64_t *bad) {
  if (workers < 1) workers = 1;
  if (workers > 256) workers = 256;
  ds_node **heads = (ds_node **)calloc(nbuckets, sizeof(ds_node *));
  ds_job jobs[256];
  pthread_t th[256];
  *bad = 0;
  double timed = 0;
  const int ops[6] = {0, 1, 4, 2, 3, 5};
  for (int k = 0; k < 6; ++k) {
    const int op = ops[k];
    const uint64_t items = (op == 4 || op == 5) ? nbuckets : n;
    const double t0 = now_s();
    for (int w = 0; w < workers; ++w) {
      jobs[w].heads = heads;
      jobs[w].nbuckets = nbuckets;
      jobs[w].tseed = tseed;
      jobs[w].kseed = kseed;
      jobs[w].op = op;
      jobs[w].bad = 0;
      jobs[w].begin = items * (uint64_t)w / (uint64_t)workers;
      jobs[w].end = items * (uint64_t)(w + 1) / (uint64_t)workers;
      pthread_create(&th[w], NULL, ds_run, &jobs[w]);
    }
    for (int w = 0; w < workers; ++w) {
      pthread_join(th[w], NULL);
      *bad += jobs[w].bad;
    }
    if (k < 4) timed += now_s() - t0;
  }
  free(heads);
  return timed;
}

typedef struct {
  const uint32_t *lengths;
  uint64_t begin, end, bad, pushes;
  uint32_t start;
} vec_job;

static void *vec_run(void *arg) {
  vec_job *j = (vec_job *)arg;
  for (uint64_t v = j->begin; v < j->end; ++v) {
    uint64_t cap = 1;
    while (cap < j->start) cap <<= 1;
    uint64_t size = 0;
    uint32_t *data = (uint32_t *)malloc(cap * 4);
    for (uint32_t i = 0; i < j->lengths[v] && data; ++i) {
      if (size == cap) {
        uint32_t *nd = (uint32_t *)malloc(cap * 8);
        if (!nd) {
          j->bad++;
          break;
        }
        memcpy(nd, data, size * 4);
        free(data);
        data = nd;
        cap *= 2;
      }
      data[size++] = (uint32_t)(v * 2654435761ull + i);
      j->pushes++;
    }
    for (uint64_t i = 0; i < size; ++i) j->bad += data[i] != (uint32_t)(v * 2654435761ull + i);
    free(data);
  }
  return NULL;
}

/* The vector-growth run with glibc; returns seconds. */
double cpu_vectors(const uint32_t *lengths, uint64_t n, uint32_t start, int workers, uint64_t *bad,
                   uint64_t *pushes) {
  if (workers < 1) workers = 1;
  if (workers > 256) workers = 256;
  vec_job jobs[256];
  pthread_t th[256];
  const double t0 = now_s();
  for (int w = 0; w < workers; ++w) {
    jobs[w].lengths = lengths;
    jobs[w].start = start;
    jobs[w].bad = jobs[w].pushes = 0;
    jobs[w].begin = n * (uint64_t)w / (uint64_t)workers;
    jobs[w].end = n * (uint64_t)(w + 1) / (uint64_t)workers;
    pthread_create(&th[w], NULL, vec_run, &jobs[w]);
  }
  *bad = *pushes = 0;
  for (int w = 0; w < workers; ++w) {
    pthread_join(th[w], NULL);
    *bad += jobs[w].bad;
    *pushes += jobs[w].pushes;
  }
  return now_s() - t0;
}
