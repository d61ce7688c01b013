// Bounded lock-free multi-producer multi-consumer ring (host side).
//
// Each cell carries a sequence number: a producer claims position p by a CAS
// on the enqueue counter when cell p % capacity shows sequence p, writes the
// value, then publishes sequence p + 1; a consumer claims position p when the
// cell shows p + 1 and frees it by publishing p + capacity.  Push and pop fail
// (return false) instead of waiting when the ring is full or empty.  This is
// D. Vyukov's bounded MPMC queue; capacity is a power of two.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <memory>

namespace bepugpu {

template <class T>
class Ring {
  public:
    explicit Ring(size_t capacity) : mask_(capacity - 1), cells_(new Cell[capacity]) {
        for (size_t i = 0; i < capacity; i++) cells_[i].seq.store(i, std::memory_order_relaxed);
        head_.store(0, std::memory_order_relaxed);
        tail_.store(0, std::memory_order_relaxed);
    }
    static bool ValidCapacity(size_t c) { return c >= 2 && (c & (c - 1)) == 0; }
    size_t Capacity() const { return mask_ + 1; }

    bool Push(const T& v) {
        size_t pos = tail_.load(std::memory_order_relaxed);
        for (;;) {
            Cell& c = cells_[pos & mask_];
            size_t seq = c.seq.load(std::memory_order_acquire);
            intptr_t dif = (intptr_t)seq - (intptr_t)pos;
            if (dif == 0) {
                if (tail_.compare_exchange_weak(pos, pos + 1, std::memory_order_relaxed)) {
                    c.value = v;
                    c.seq.store(pos + 1, std::memory_order_release);
                    return true;
                }
            } else if (dif < 0) {
                return false;  // full
            } else {
                pos = tail_.load(std::memory_order_relaxed);
            }
        }
    }
    bool Pop(T& out) {
        size_t pos = head_.load(std::memory_order_relaxed);
        for (;;) {
            Cell& c = cells_[pos & mask_];
            size_t seq = c.seq.load(std::memory_order_acquire);
            intptr_t dif = (intptr_t)seq - (intptr_t)(pos + 1);
            if (dif == 0) {
                if (head_.compare_exchange_weak(pos, pos + 1, std::memory_order_relaxed)) {
                    out = c.value;
                    c.seq.store(pos + mask_ + 1, std::memory_order_release);
                    return true;
                }
            } else if (dif < 0) {
                return false;  // empty
            } else {
                pos = head_.load(std::memory_order_relaxed);
            }
        }
    }

  private:
    struct Cell {
        std::atomic<size_t> seq;
        T value;
    };
    const size_t mask_;
    std::unique_ptr<Cell[]> cells_;
    alignas(64) std::atomic<size_t> tail_;
    alignas(64) std::atomic<size_t> head_;
};

}  // namespace bepugpu
