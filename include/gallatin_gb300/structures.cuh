// Allocator-backed device data structures: a chained hash table whose nodes
// come from the allocator, and a per-thread doubling vector. They follow the
// reference's chaining_table / chaining_block (data_structs/
// chaining_table.cuh:57-327) and svector (data_structs/single_vector.cuh:
// 50-200): the same node shape (next pointer, N keys, N values), the same
// bucket choice (MurmurHash64A of the key mod the bucket count), the same
// append-a-node-on-overflow insert, and the same malloc-copy-free doubling.
// Added here: erase (the reference table has none) and a compaction pass that
// unlinks and frees nodes whose keys were all erased.
//
// Both are templates over the allocator type A (anything with device
// malloc(bytes) / free(ptr)), so the same code runs over this library's
// allocator and over others. Every loop is bounded. The table's insert is
// force-inlined: compiled as a call, it put a 152-byte stack frame and
// register saves around every insert. The vector's growth stays
// a call: inlined into push_back's loop it raised the loop's spills and the
// vectors ran 29 % slower.
//
// Concurrency: inserts, erases and queries of distinct keys may run at once.
// A query that races an insert of the same key can see the key before its
// value; erase and insert of the same key at once is undefined. compact() and
// clear() need the bucket to themselves.
#ifndef GALLATIN_GB300_STRUCTURES_CUH
#define GALLATIN_GB300_STRUCTURES_CUH

#include <stdint.h>

#include "murmur.cuh"

namespace galds {

constexpr uint64_t kEmptyKey = ~0ull;  // never inserted (reference defaultKey)
constexpr int kMaxChain = 1 << 16;     // nodes walked per operation at most

template <int N = 7>
struct chaining_block {
  chaining_block *next;
  uint64_t keys[N];
  uint64_t vals[N];

  __device__ void init() {
    next = nullptr;
    for (int i = 0; i < N; ++i) keys[i] = kEmptyKey;
  }
  __device__ bool empty() const {
    for (int i = 0; i < N; ++i)
      if (keys[i] != kEmptyKey) return false;
    return true;
  }
};
static_assert(sizeof(chaining_block<7>) == 120, "a 7-slot node is 120 B: it takes one 128 B slice");

template <class A, int N = 7>
struct chaining_table {
  using block_type = chaining_block<N>;
  A *alloc;
  block_type **heads;  // [nbuckets], device memory the owner provides, zeroed
  uint64_t nbuckets;
  uint64_t seed;

  __device__ uint64_t bucket(uint64_t key) const { return gal::murmur64a_u64(key, seed) % nbuckets; }

  // a link as other threads last published it (not a stale L1 copy)
  __device__ static block_type *load_link(block_type *const *link) {
    return *(block_type *const volatile *)link;
  }

  // Insert key -> val. Returns false only when a node was needed and the
  // allocator returned NULL (or the chain bound was hit).
  __device__ __forceinline__ bool insert(uint64_t key, uint64_t val) {
    block_type **link = heads + bucket(key);
    block_type *b = load_link(link);
    for (int hop = 0; hop < kMaxChain; ++hop) {
      if (b == nullptr) {
        block_type *nb = (block_type *)alloc->malloc(sizeof(block_type));
        if (nb == nullptr) return false;
        nb->init();
        __threadfence();  // the node's contents before its publication
        block_type *prev = (block_type *)atomicCAS((unsigned long long *)link, 0ull, (unsigned long long)nb);
        if (prev != nullptr) {  // another thread appended first: use its node
          alloc->free(nb);
          b = prev;
        } else {
          b = nb;
        }
      }
      for (int i = 0; i < N; ++i) {
        if (b->keys[i] == kEmptyKey &&
            atomicCAS((unsigned long long *)&b->keys[i], kEmptyKey, (unsigned long long)key) == kEmptyKey) {
          b->vals[i] = val;
          return true;
        }
      }
      link = &b->next;
      b = load_link(link);
    }
    return false;
  }

  __device__ bool query(uint64_t key, uint64_t &val) const {
    const block_type *b = heads[bucket(key)];
    for (int hop = 0; hop < kMaxChain && b != nullptr; ++hop) {
      for (int i = 0; i < N; ++i) {
        if (b->keys[i] == key) {
          val = b->vals[i];
          return true;
        }
      }
      b = b->next;
    }
    return false;
  }

  // Erase key; its slot can be reused by a later insert. False if absent.
  __device__ bool erase(uint64_t key) {
    block_type *b = heads[bucket(key)];
    for (int hop = 0; hop < kMaxChain && b != nullptr; ++hop) {
      for (int i = 0; i < N; ++i) {
        if (b->keys[i] == key &&
            atomicCAS((unsigned long long *)&b->keys[i], (unsigned long long)key, kEmptyKey) == key)
          return true;
      }
      b = b->next;
    }
    return false;
  }

  // Unlink and free the nodes of bucket i that hold no key; returns how many.
  __device__ uint32_t compact(uint64_t i) {
    uint32_t freed = 0;
    block_type **link = heads + i;
    for (int hop = 0; hop < kMaxChain && *link != nullptr; ++hop) {
      block_type *b = *link;
      if (b->empty()) {
        *link = b->next;
        alloc->free(b);
        ++freed;
      } else {
        link = &b->next;
      }
    }
    return freed;
  }

  // Free every node of bucket i; returns how many.
  __device__ uint32_t clear(uint64_t i) {
    uint32_t freed = 0;
    block_type *b = heads[i];
    for (int hop = 0; hop < kMaxChain && b != nullptr; ++hop) {
      block_type *next = b->next;
      alloc->free(b);
      ++freed;
      b = next;
    }
    heads[i] = nullptr;
    return freed;
  }

  __device__ uint32_t chain_length(uint64_t i) const {
    uint32_t n = 0;
    for (const block_type *b = heads[i]; b != nullptr && n < (uint32_t)kMaxChain; b = b->next) ++n;
    return n;
  }
};

// A vector owned by one thread, grown by doubling: a new backing of twice
// the size is allocated, the items copied and the old backing freed.
template <class T, class A>
struct svector {
  uint64_t size;
  uint64_t backing_size;
  T *data;
  A *alloc;

  // Backing for the first `starting_count` items, rounded up to a power of
  // two (reference svector(starting_count)). False if the allocator had none.
  __device__ bool init(A *a, uint64_t starting_count) {
    alloc = a;
    uint64_t n = 1;
    while (n < starting_count) n <<= 1;
    backing_size = n;
    size = 0;
    data = (T *)alloc->malloc(sizeof(T) * n);
    return data != nullptr;
  }

  __device__ bool upsize() {
    const uint64_t bytes = sizeof(T) * size;
    T *nd = (T *)alloc->malloc(sizeof(T) * backing_size * 2);
    if (nd == nullptr) return false;
    // both backings are allocator blocks, 16-byte aligned: copy 16 B at a time
    const uint4 *src = (const uint4 *)data;
    uint4 *dst = (uint4 *)nd;
    const uint64_t vec = bytes / 16;
    for (uint64_t k = 0; k < vec; ++k) dst[k] = src[k];
    for (uint64_t k = vec * 16; k < bytes; ++k) ((char *)nd)[k] = ((const char *)data)[k];
    alloc->free(data);
    data = nd;
    backing_size *= 2;
    return true;
  }

  __device__ bool push_back(T item) {
    if (size == backing_size && !upsize()) return false;
    data[size++] = item;
    return true;
  }

  __device__ T &operator[](uint64_t i) { return data[i]; }
  __device__ const T &operator[](uint64_t i) const { return data[i]; }

  __device__ void free_vector() {
    if (data) alloc->free(data);
    data = nullptr;
    size = backing_size = 0;
  }
};

}  // namespace galds

#endif  // GALLATIN_GB300_STRUCTURES_CUH
