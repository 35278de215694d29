// UnorderedMap and Bitset of the header path, with the reference's names and
// semantics (containers/src/Kokkos_UnorderedMap.hpp:50-960,
// containers/src/Kokkos_Bitset.hpp:49-300).
//
// UnorderedMap layout: a power-of-two table of slots (keys, values and one
// 32-bit state word per slot: empty, being written, valid, erased) with
// linear probing from a 64-bit finaliser hash of the key.  An insert claims
// an empty slot with one compare-and-swap on its state word, writes key and
// value, and publishes the slot with a release store; an insert or find that
// meets a slot being written waits for it (bounded) and then compares keys,
// so a key is valid in at most one slot.  Erased slots stay tombstones until
// clear() or rehash(); they are skipped by find and never reclaimed by
// insert, which keeps concurrent inserts of one key consistent.  The
// reference threads its entries through per-bucket linked lists instead;
// only the API and the result semantics are the same: insert returns
// success / existing / failed with the entry's index, find returns the index
// or invalid_index, and failed_insert() reports a full table.
#pragma once

#include <cstring>

#include "scan.hpp"

namespace gb300k {

constexpr uint32_t UnorderedMapInvalidIndex = ~0u;

// insert() result (Kokkos_UnorderedMap.hpp:85-140).
class UnorderedMapInsertResult {
 public:
  KOKKOS_FORCEINLINE_FUNCTION bool success() const { return status_ == kSuccess; }
  KOKKOS_FORCEINLINE_FUNCTION bool existing() const { return status_ == kExisting; }
  KOKKOS_FORCEINLINE_FUNCTION bool failed() const { return index_ == UnorderedMapInvalidIndex; }
  KOKKOS_FORCEINLINE_FUNCTION bool freed_existing() const { return false; }
  KOKKOS_FORCEINLINE_FUNCTION uint32_t list_position() const { return probes_; }
  KOKKOS_FORCEINLINE_FUNCTION uint32_t index() const { return index_; }
  KOKKOS_FORCEINLINE_FUNCTION UnorderedMapInsertResult() {}
  KOKKOS_FORCEINLINE_FUNCTION UnorderedMapInsertResult(uint32_t index, uint32_t status, uint32_t probes)
      : index_(index), status_(status), probes_(probes) {}
  static constexpr uint32_t kSuccess = 1, kExisting = 2;

 private:
  uint32_t index_ = UnorderedMapInvalidIndex, status_ = 0, probes_ = 0;
};

// What an insert of an existing key does with its value
// (Kokkos_UnorderedMap.hpp:150-171): NoOp keeps the first value, AtomicAdd
// adds the new one.
template <class ValueTypeView, class ValuesIdxType = uint32_t>
struct UnorderedMapInsertOpTypes {
  using value_type = std::remove_const_t<typename ValueTypeView::value_type>;
  struct NoOp {
    KOKKOS_FUNCTION void op(const ValueTypeView&, ValuesIdxType, const value_type&) const {}
  };
  struct AtomicAdd {
    KOKKOS_FUNCTION void op(const ValueTypeView& values, ValuesIdxType i, const value_type& v) const {
#ifdef __CUDA_ARCH__
      Impl::atomic_add_old(values.data() + i, v);
#else
      values.data()[i] += v;
#endif
    }
  };
};

namespace Impl {
// 64-bit finaliser (Stafford's variant 13 of the MurmurHash3 fmix64 mixer)
// over the key's bytes folded 8 at a time.
template <class K>
struct pod_hash {
  KOKKOS_INLINE_FUNCTION uint64_t operator()(const K& k) const {
    uint64_t h = 0x9E3779B97F4A7C15ull * (sizeof(K) + 1);
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&k);
    for (size_t o = 0; o < sizeof(K); o += 8) {
      uint64_t w = 0;
      const size_t m = sizeof(K) - o < 8 ? sizeof(K) - o : 8;
      for (size_t b = 0; b < m; ++b) w |= (uint64_t)p[o + b] << (8 * b);
      h ^= w;
      h ^= h >> 30;
      h *= 0xBF58476D1CE4E5B9ull;
      h ^= h >> 27;
      h *= 0x94D049BB133111EBull;
      h ^= h >> 31;
    }
    return h;
  }
};
// Key equality by bytes (the reference's pod_equal_to).
template <class K>
struct pod_equal_to {
  KOKKOS_INLINE_FUNCTION bool operator()(const K& a, const K& b) const {
    const unsigned char* x = reinterpret_cast<const unsigned char*>(&a);
    const unsigned char* y = reinterpret_cast<const unsigned char*>(&b);
    for (size_t i = 0; i < sizeof(K); ++i)
      if (x[i] != y[i]) return false;
    return true;
  }
};

constexpr uint32_t kSlotEmpty = 0, kSlotBusy = 1, kSlotValid = 2, kSlotErased = 3;
// An insert places a key within this many slots of its hash position, so a
// find stops there too (the reference's bounded insert); a table that has no
// free slot in that window reports a failed insert.
constexpr uint32_t kMaxProbes = 4096;
// scalars: [0] size, [1] failed-insert flag, [2] erase enabled, [3] wait gave up
constexpr int kMapScalars = 4;
}  // namespace Impl

template <class Key, class Value, class Device = Experimental::GB300, class Hasher = Impl::pod_hash<Key>,
          class EqualTo = Impl::pod_equal_to<Key>>
class UnorderedMap {
 public:
  using key_type = Key;
  using value_type = Value;
  using size_type = uint32_t;
  using hasher_type = Hasher;
  using equal_to_type = EqualTo;
  static constexpr bool is_set = std::is_void<Value>::value;
  using impl_value_type = std::conditional_t<is_set, int, Value>;
  using values_view = View<impl_value_type*>;
  using insert_result = UnorderedMapInsertResult;
  using default_op_type = typename UnorderedMapInsertOpTypes<values_view, uint32_t>::NoOp;
  static constexpr bool is_insertable_map = true;
  static constexpr size_type invalid_index = UnorderedMapInvalidIndex;

  UnorderedMap() = default;
  // capacity() >= capacity_hint: the next power of two at or above 4/3 of
  // the hint (a table at most three quarters full when the hint is met).
  explicit UnorderedMap(size_type capacity_hint, Hasher h = Hasher(), EqualTo eq = EqualTo())
      : hasher_(h), equal_(eq) {
    allocate(capacity_for(capacity_hint));
  }

  // ---- host ------------------------------------------------------------
  KOKKOS_INLINE_FUNCTION size_type capacity() const { return cap_; }
  KOKKOS_INLINE_FUNCTION size_type hash_capacity() const { return cap_; }
  size_type size() const { return (size_type)read_scalar(0); }
  bool failed_insert() const { return read_scalar(1) != 0 || read_scalar(3) != 0; }
  void reset_failed_insert_flag() {
    write_scalar(1, 0);
    write_scalar(3, 0);
  }
  // Every entry removed, the capacity kept.
  void clear() {
    if (!cap_) return;
    check_cuda(cudaMemset(state_.data(), 0, sizeof(uint32_t) * cap_), "UnorderedMap::clear");
    check_cuda(cudaMemset(scalars_.data(), 0, sizeof(uint32_t) * Impl::kMapScalars), "UnorderedMap::clear");
  }
  // erase() takes effect only between begin_erase() and end_erase()
  // (Kokkos_UnorderedMap.hpp:490-515).
  bool begin_erase() {
    write_scalar(2, 1);
    return true;
  }
  bool end_erase() {
    check_cuda(cudaDeviceSynchronize(), "UnorderedMap::end_erase");
    write_scalar(2, 0);
    return true;
  }
  // A table of at least max(requested, size()) capacity holding the same
  // entries; returns true on success (Kokkos_UnorderedMap.hpp:437-468).
  bool rehash(size_type requested_capacity = 0);

  // ---- device ----------------------------------------------------------
  template <class InsertOp = default_op_type>
  KOKKOS_INLINE_FUNCTION insert_result insert(const Key& k, const impl_value_type& v = impl_value_type(),
                                              InsertOp op = InsertOp()) const {
#ifdef __CUDA_ARCH__
    if (!cap_) return insert_result();
    const uint32_t mask = cap_ - 1;
    uint32_t i = (uint32_t)hasher_(k) & mask;
    const uint32_t probes = cap_ < Impl::kMaxProbes ? cap_ : Impl::kMaxProbes;
    for (uint32_t p = 0; p < probes; ++p, i = (i + 1) & mask) {
      uint32_t s = gbk::ld_acquire_u32(state_.data() + i);
      if (s == Impl::kSlotEmpty) {
        s = atomicCAS(state_.data() + i, Impl::kSlotEmpty, Impl::kSlotBusy);
        if (s == Impl::kSlotEmpty) {
          keys_.data()[i] = k;
          if (!is_set) values_.data()[i] = v;
          gbk::st_release_u32(state_.data() + i, Impl::kSlotValid);  // orders the key and value before it
          count_size(1);
          return insert_result(i, insert_result::kSuccess, p);
        }
      }
      if (s == Impl::kSlotBusy && !wait_valid(i, &s)) return insert_result();
      if (s == Impl::kSlotValid && equal_(keys_.data()[i], k)) {
        if (!is_set) op.op(values_, i, v);
        return insert_result(i, insert_result::kExisting, p);
      }
    }
    atomicOr(scalars_.data() + 1, 1u);
    return insert_result();
#else
    (void)k;
    (void)v;
    (void)op;
    return insert_result();
#endif
  }
  KOKKOS_INLINE_FUNCTION size_type find(const Key& k) const {
#ifdef __CUDA_ARCH__
    if (!cap_) return invalid_index;
    const uint32_t mask = cap_ - 1;
    uint32_t i = (uint32_t)hasher_(k) & mask;
    const uint32_t probes = cap_ < Impl::kMaxProbes ? cap_ : Impl::kMaxProbes;
    for (uint32_t p = 0; p < probes; ++p, i = (i + 1) & mask) {
      uint32_t s = gbk::ld_acquire_u32(state_.data() + i);
      if (s == Impl::kSlotEmpty) return invalid_index;
      if (s == Impl::kSlotBusy && !wait_valid(i, &s)) return invalid_index;
      if (s == Impl::kSlotValid && equal_(keys_.data()[i], k)) return i;
    }
    return invalid_index;
#else
    (void)k;
    return invalid_index;
#endif
  }
  KOKKOS_INLINE_FUNCTION bool exists(const Key& k) const { return valid_at(find(k)); }
  KOKKOS_INLINE_FUNCTION bool valid_at(size_type i) const {
#ifdef __CUDA_ARCH__
    return i < cap_ && gbk::ld_acquire_u32(state_.data() + i) == Impl::kSlotValid;
#else
    (void)i;
    return false;
#endif
  }
  KOKKOS_FORCEINLINE_FUNCTION Key key_at(size_type i) const { return keys_.data()[i]; }
  template <class D = Value, std::enable_if_t<!std::is_void<D>::value, bool> = true>
  KOKKOS_FORCEINLINE_FUNCTION impl_value_type& value_at(size_type i) const {
    return values_.data()[i];
  }
  // Remove k (between begin_erase and end_erase); true if it was present.
  KOKKOS_INLINE_FUNCTION bool erase(const Key& k) const {
#ifdef __CUDA_ARCH__
    if (!cap_ || !*(volatile uint32_t*)(scalars_.data() + 2)) return false;
    const uint32_t i = find(k);
    if (i == invalid_index) return false;
    if (atomicCAS(state_.data() + i, Impl::kSlotValid, Impl::kSlotErased) != Impl::kSlotValid) return false;
    count_size(-1);
    return true;
#else
    (void)k;
    return false;
#endif
  }

  // (rehash kernel access)
  const View<Key*>& impl_keys() const { return keys_; }
  const values_view& impl_values() const { return values_; }
  const View<uint32_t*>& impl_state() const { return state_; }

 private:
  static size_type capacity_for(size_type hint) {
    uint64_t want = (uint64_t)hint + hint / 3;
    uint64_t c = 128;
    while (c < want) c <<= 1;
    if (c > (1ull << 31)) throw std::runtime_error("UnorderedMap: capacity above 2^31");
    return (size_type)c;
  }
  void allocate(size_type cap) {
    cap_ = cap;
    keys_ = View<Key*>("UnorderedMap keys", cap);
    values_ = values_view("UnorderedMap values", is_set ? 0 : cap);
    state_ = View<uint32_t*>("UnorderedMap state", cap);
    scalars_ = View<uint32_t*>("UnorderedMap scalars", Impl::kMapScalars);
  }
  uint32_t read_scalar(int k) const {
    if (!cap_) return 0;
    uint32_t v = 0;
    check_cuda(cudaDeviceSynchronize(), "UnorderedMap");
    check_cuda(cudaMemcpy(&v, scalars_.data() + k, 4, cudaMemcpyDeviceToHost), "UnorderedMap");
    return v;
  }
  void write_scalar(int k, uint32_t v) {
    if (!cap_) return;
    check_cuda(cudaDeviceSynchronize(), "UnorderedMap");
    check_cuda(cudaMemcpy(scalars_.data() + k, &v, 4, cudaMemcpyHostToDevice), "UnorderedMap");
  }
#ifdef __CUDA_ARCH__
  // size += d for every lane of the warp that reaches this call together:
  // one atomic per group of lanes instead of one per entry, so inserts of
  // distinct keys do not serialise on the one size word.
  __device__ void count_size(int d) const {
    const unsigned g = __activemask();
    const int lead = __ffs(g) - 1;
    if ((int)(threadIdx.x & 31) == lead) atomicAdd(scalars_.data() + 0, (uint32_t)(d * __popc(g)));
  }
  // A slot being written by another insert: wait (bounded) until it is
  // published; on a wait that gives up, record it and report failure.
  __device__ bool wait_valid(uint32_t i, uint32_t* s) const {
    for (int64_t polls = 0; polls < ((int64_t)1 << 22); ++polls) {
      *s = gbk::ld_acquire_u32(state_.data() + i);
      if (*s != Impl::kSlotBusy) return true;
      if (polls > 16) __nanosleep(64);
    }
    atomicOr(scalars_.data() + 3, 1u);
    return false;
  }
#endif

  size_type cap_ = 0;
  Hasher hasher_{};
  EqualTo equal_{};
  View<Key*> keys_;
  values_view values_;
  View<uint32_t*> state_;
  View<uint32_t*> scalars_;
};

namespace Impl {
template <class Map>
__global__ void k_umap_rehash(Map src, Map dst) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= src.capacity() || !src.valid_at(i)) return;
  if constexpr (Map::is_set) {
    dst.insert(src.key_at(i));
  } else {
    dst.insert(src.key_at(i), src.value_at(i));
  }
}
}  // namespace Impl

template <class Key, class Value, class Device, class Hasher, class EqualTo>
bool UnorderedMap<Key, Value, Device, Hasher, EqualTo>::rehash(size_type requested_capacity) {
  const size_type n = size();
  const size_type want = requested_capacity > n ? requested_capacity : n;
  UnorderedMap next(want, hasher_, equal_);
  if (cap_) {
    Impl::k_umap_rehash<<<(cap_ + 255) / 256, 256>>>(*this, next);
    Impl::launched(cudaGetLastError(), "UnorderedMap::rehash");
    check_cuda(cudaDeviceSynchronize(), "UnorderedMap::rehash");
    if (next.failed_insert()) return false;
  }
  *this = next;
  return true;
}

// ---- Bitset (containers/src/Kokkos_Bitset.hpp:49-300) ------------------------
namespace Impl {
struct BitsetPopc {
  const uint32_t* b;
  int64_t nb;
  uint32_t lm;  // valid bits of the last block (0: all)
  __device__ void operator()(int64_t i, unsigned& u) const {
    uint32_t w = b[i];
    if (i == nb - 1 && lm) w &= lm;
    u += (unsigned)__popc(w);
  }
};
}  // namespace Impl

template <class Device = Experimental::GB300>
class Bitset {
 public:
  static constexpr unsigned BIT_SCAN_REVERSE = 1u;
  static constexpr unsigned MOVE_HINT_BACKWARD = 2u;
  static constexpr unsigned BIT_SCAN_FORWARD_MOVE_HINT_FORWARD = 0u;
  static constexpr unsigned BIT_SCAN_REVERSE_MOVE_HINT_FORWARD = BIT_SCAN_REVERSE;
  static constexpr unsigned BIT_SCAN_FORWARD_MOVE_HINT_BACKWARD = MOVE_HINT_BACKWARD;
  static constexpr unsigned BIT_SCAN_REVERSE_MOVE_HINT_BACKWARD = BIT_SCAN_REVERSE | MOVE_HINT_BACKWARD;

  Bitset() = default;
  explicit Bitset(unsigned arg_size)
      : size_(arg_size), blocks_("Bitset", (arg_size + 31) / 32), last_mask_(arg_size % 32 ? (1u << (arg_size % 32)) - 1u : 0u) {}

  KOKKOS_FORCEINLINE_FUNCTION unsigned size() const { return size_; }
  // Number of set bits (a header reduce of popc over the blocks).
  unsigned count() const {
    if (!size_) return 0;
    unsigned c = 0;
    const uint32_t* b = blocks_.data();
    const int64_t nb = (int64_t)blocks_.size();
    const uint32_t lm = last_mask_;
    parallel_reduce(RangePolicy<>(0, nb), Impl::BitsetPopc{b, nb, lm}, c);
    return c;
  }
  void set() {
    if (!size_) return;
    const uint32_t ones = ~0u;
    check(gbk_fill(blocks_.data(), &ones, 4, (int64_t)blocks_.size(), nullptr), "Bitset::set");
    if (last_mask_) {
      const uint32_t lm = last_mask_;
      check(gbk_fill(blocks_.data() + blocks_.size() - 1, &lm, 4, 1, nullptr), "Bitset::set");
    }
    check_cuda(cudaStreamSynchronize(nullptr), "Bitset::set");
  }
  void reset() {
    if (!size_) return;
    check_cuda(cudaMemset(blocks_.data(), 0, 4 * blocks_.size()), "Bitset::reset");
  }
  void clear() { reset(); }

  // true if this call changed the bit (atomic)
  KOKKOS_FORCEINLINE_FUNCTION bool set(unsigned i) const {
#ifdef __CUDA_ARCH__
    if (i >= size_) return false;
    const uint32_t m = 1u << (i & 31);
    return !(atomicOr(blocks_.data() + (i >> 5), m) & m);
#else
    (void)i;
    return false;
#endif
  }
  KOKKOS_FORCEINLINE_FUNCTION bool reset(unsigned i) const {
#ifdef __CUDA_ARCH__
    if (i >= size_) return false;
    const uint32_t m = 1u << (i & 31);
    return atomicAnd(blocks_.data() + (i >> 5), ~m) & m;
#else
    (void)i;
    return false;
#endif
  }
  KOKKOS_FORCEINLINE_FUNCTION bool test(unsigned i) const {
#ifdef __CUDA_ARCH__
    if (i >= size_) return false;
    return (*(volatile uint32_t*)(blocks_.data() + (i >> 5)) >> (i & 31)) & 1u;
#else
    (void)i;
    return false;
#endif
  }
  KOKKOS_FORCEINLINE_FUNCTION unsigned max_hint() const { return (unsigned)blocks_.size(); }
  // A set (unset) bit in the 32-bit block of the hint: {true, bit}, else
  // {false, a hint into the next block in the scan direction}.  Forward scans
  // return the first such bit at or after the hint's position in its block
  // (wrapping inside the block), reverse scans the last at or before it.
  KOKKOS_INLINE_FUNCTION pair<bool, unsigned> find_any_set_near(
      unsigned hint, unsigned dir = BIT_SCAN_FORWARD_MOVE_HINT_FORWARD) const {
    return find_near(hint, dir, false);
  }
  KOKKOS_INLINE_FUNCTION pair<bool, unsigned> find_any_unset_near(
      unsigned hint, unsigned dir = BIT_SCAN_FORWARD_MOVE_HINT_FORWARD) const {
    return find_near(hint, dir, true);
  }

 private:
  KOKKOS_INLINE_FUNCTION pair<bool, unsigned> find_near(unsigned hint, unsigned dir, bool unset) const {
#ifdef __CUDA_ARCH__
    const unsigned nb = (unsigned)blocks_.size();
    if (!nb) return {false, 0u};
    const unsigned bi = (hint >> 5) < nb ? (hint >> 5) : 0;
    const unsigned off = hint & 31;
    uint32_t w = *(volatile uint32_t*)(blocks_.data() + bi);
    if (unset) w = ~w;
    if (bi == nb - 1 && last_mask_) w &= last_mask_;
    if (w) {
      unsigned bit;
      if (!(dir & BIT_SCAN_REVERSE)) {
        const uint32_t hi = w & (~0u << off);
        bit = hi ? __ffs(hi) - 1 : __ffs(w) - 1;
      } else {
        const uint32_t lo = off == 31 ? w : w & ((2u << off) - 1u);
        bit = lo ? 31 - __clz(lo) : 31 - __clz(w);
      }
      return {true, bi * 32 + bit};
    }
    const unsigned next = (dir & MOVE_HINT_BACKWARD) ? (bi == 0 ? nb - 1 : bi - 1) : (bi + 1 == nb ? 0 : bi + 1);
    return {false, next * 32};
#else
    (void)hint;
    (void)dir;
    (void)unset;
    return {false, 0u};
#endif
  }

  unsigned size_ = 0;
  View<uint32_t*> blocks_;
  uint32_t last_mask_ = 0;
};

}  // namespace gb300k
