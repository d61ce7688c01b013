// Device memory for scene arenas and staging buffers (host code).
//
// A context's scenes take their arenas from a few large cudaMalloc slabs,
// best fit with coalescing, so creating, destroying, spilling and restoring a
// scene moves heap blocks instead of calling the CUDA allocator: a spill or a
// restore never waits for the device, and thousands of served scenes map a
// handful of slabs rather than one allocation each.
//
// A block freed while work queued on a stream may still read it (a spill's
// copy) is parked with an event recorded on that stream and becomes
// allocatable once the event has completed.

#include <cuda_runtime.h>

#include <algorithm>

#include "bepugpu_internal.h"

namespace bepugpu {

namespace {
constexpr size_t kAlign = 256;
constexpr size_t kMinSlab = 64ull << 20;
constexpr size_t kMaxSlab = 1ull << 30;
constexpr size_t kSlabGranule = 2ull << 20;
size_t RoundUp(size_t x, size_t a) { return (x + a - 1) / a * a; }
}  // namespace

DeviceHeap::~DeviceHeap() {
    for (Pending& p : pending_) cudaEventDestroy(p.done);
    for (cudaEvent_t e : spareEvents_) cudaEventDestroy(e);
    for (Slab& s : slabs_) cudaFree(s.base);
}

void DeviceHeap::InsertFree(char* p, size_t bytes, int slab) {
    // coalesce with the free neighbours of the same slab
    auto next = free_.lower_bound(p);
    if (next != free_.end() && next->first == p + bytes && next->second.slab == slab) {
        bytes += next->second.bytes;
        EraseSized(next->first, next->second.bytes);
        next = free_.erase(next);
    }
    if (next != free_.begin()) {
        auto prev = std::prev(next);
        if (prev->first + prev->second.bytes == p && prev->second.slab == slab) {
            p = prev->first;
            bytes += prev->second.bytes;
            EraseSized(prev->first, prev->second.bytes);
            free_.erase(prev);
        }
    }
    free_[p] = FreeRange{bytes, slab};
    bySize_.emplace(bytes, p);
}

void DeviceHeap::EraseSized(char* p, size_t bytes) {
    auto range = bySize_.equal_range(bytes);
    for (auto it = range.first; it != range.second; ++it)
        if (it->second == p) {
            bySize_.erase(it);
            return;
        }
}

void DeviceHeap::Reclaim(bool wait) {
    for (auto it = pending_.begin(); it != pending_.end();) {
        cudaError_t e = wait ? cudaEventSynchronize(it->done) : cudaEventQuery(it->done);
        if (e == cudaErrorNotReady) {
            ++it;
            continue;
        }
        // on a failed stream the copy is over too: the block is not read any more
        spareEvents_.push_back(it->done);
        ReleaseBlock(it->p);
        it = pending_.erase(it);
    }
}

void DeviceHeap::ReleaseBlock(char* p) {
    auto it = live_.find(p);
    if (it == live_.end()) return;
    const size_t bytes = it->second.bytes;
    const int slab = it->second.slab;
    live_.erase(it);
    inUse_ -= bytes;
    InsertFree(p, bytes, slab);
    if (holds_ == 0) TrimEmptySlabs();
}

void DeviceHeap::TrimEmptySlabs() {
    for (size_t i = 0; i < slabs_.size(); i++) {
        Slab& s = slabs_[i];
        if (!s.base) continue;
        auto it = free_.find(s.base);
        if (it == free_.end() || it->second.bytes != s.bytes) continue;
        EraseSized(it->first, it->second.bytes);
        free_.erase(it);
        cudaFree(s.base);
        reserved_ -= s.bytes;
        s.base = nullptr;  // slab indices of the other ranges stay valid
        s.bytes = 0;
    }
}

cudaError_t DeviceHeap::Alloc(size_t bytes, void** out) {
    std::lock_guard<std::mutex> g(mu_);
    *out = nullptr;
    bytes = RoundUp(std::max<size_t>(bytes, 1), kAlign);
    Reclaim(false);
    for (int attempt = 0; attempt < 2; attempt++) {
        auto it = bySize_.lower_bound(bytes);
        if (it != bySize_.end()) {
            char* p = it->second;
            const size_t have = it->first;
            bySize_.erase(it);
            auto f = free_.find(p);
            const int slab = f->second.slab;
            free_.erase(f);
            if (have > bytes) InsertFree(p + bytes, have - bytes, slab);
            live_[p] = LiveBlock{bytes, slab};
            inUse_ += bytes;
            *out = p;
            return cudaSuccess;
        }
        if (pending_.empty()) break;
        Reclaim(true);  // blocks whose last copies are still running
    }
    // a new slab: geometric growth, and large arenas get one of their own
    size_t slabBytes = bytes >= kMaxSlab / 4 ? RoundUp(bytes, kSlabGranule)
                                             : std::min(kMaxSlab, std::max(kMinSlab, RoundUp(reserved_, kSlabGranule)));
    slabBytes = std::max(slabBytes, RoundUp(bytes, kSlabGranule));
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, slabBytes);
    if (e != cudaSuccess) {
        cudaGetLastError();  // the failed allocation is reported to the caller, not to later launches
        return e;
    }
    int slab = -1;
    for (size_t i = 0; i < slabs_.size(); i++)
        if (!slabs_[i].base) {
            slab = (int)i;
            break;
        }
    if (slab < 0) {
        slab = (int)slabs_.size();
        slabs_.push_back({});
    }
    slabs_[slab] = Slab{base, slabBytes};
    reserved_ += slabBytes;
    if (slabBytes > bytes) InsertFree(base + bytes, slabBytes - bytes, slab);
    live_[base] = LiveBlock{bytes, slab};
    inUse_ += bytes;
    *out = base;
    return cudaSuccess;
}

void DeviceHeap::Free(void* p) {
    if (!p) return;
    std::lock_guard<std::mutex> g(mu_);
    ReleaseBlock((char*)p);
}

cudaError_t DeviceHeap::FreeAfter(void* p, cudaStream_t stream) {
    if (!p) return cudaSuccess;
    std::lock_guard<std::mutex> g(mu_);
    cudaEvent_t ev = nullptr;
    if (!spareEvents_.empty()) {
        ev = spareEvents_.back();
        spareEvents_.pop_back();
    } else {
        cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaEventRecord(ev, stream);
    if (e != cudaSuccess) {
        spareEvents_.push_back(ev);
        return e;
    }
    pending_.push_back(Pending{(char*)p, ev});
    return cudaSuccess;
}

void DeviceHeap::Hold(bool hold) {
    std::lock_guard<std::mutex> g(mu_);
    if (hold) {
        holds_++;
    } else if (holds_ > 0 && --holds_ == 0) {
        Reclaim(true);
        TrimEmptySlabs();
    }
}

size_t DeviceHeap::Reserved() const {
    std::lock_guard<std::mutex> g(mu_);
    return reserved_;
}

size_t DeviceHeap::InUse() const {
    std::lock_guard<std::mutex> g(mu_);
    return inUse_;
}

}  // namespace bepugpu
