// arena.h -- a device-memory arena for shots that come and go while others run.
//
// cudaFree waits for the whole device, so a server that frees a finished shot's
// buffers with it would stall its feeding of every other shot.  The arena takes
// one cudaMalloc up front and hands out 256-byte aligned blocks first-fit from
// a free list (adjacent free blocks merge); release is host bookkeeping only.
// Callers release a shot's blocks only after its stream has finished with them.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <iterator>
#include <map>
#include <mutex>

namespace qp {

class Arena {
   public:
    Arena() = default;
    Arena(const Arena&) = delete;
    Arena& operator=(const Arena&) = delete;
    ~Arena() {
        if (base_) cudaFree(base_);
    }
    cudaError_t init(size_t bytes) {
        const cudaError_t e = cudaMalloc(&base_, bytes);
        if (e != cudaSuccess) {
            base_ = nullptr;
            return e;
        }
        cap_ = bytes;
        free_.clear();
        free_[0] = bytes;
        used_ = 0;
        return cudaSuccess;
    }
    void* alloc(size_t bytes) {
        bytes = (bytes + 255) / 256 * 256;
        if (bytes == 0) bytes = 256;
        std::lock_guard<std::mutex> lk(mu_);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, sz = it->second;
            free_.erase(it);
            if (sz > bytes) free_[off + bytes] = sz - bytes;
            taken_[off] = bytes;
            used_ += bytes;
            return base_ + off;
        }
        return nullptr;
    }
    bool owns(const void* p) const {
        return base_ && p >= (const void*)base_ && p < (const void*)(base_ + cap_);
    }
    void release(void* p) {
        if (!owns(p)) return;
        std::lock_guard<std::mutex> lk(mu_);
        const size_t off = (size_t)((char*)p - base_);
        auto t = taken_.find(off);
        if (t == taken_.end()) return;
        size_t o = off, sz = t->second;
        taken_.erase(t);
        used_ -= sz;
        auto nx = free_.lower_bound(o);
        if (nx != free_.end() && nx->first == o + sz) {  // merge with the next free block
            sz += nx->second;
            nx = free_.erase(nx);
        }
        if (nx != free_.begin()) {  // merge with the previous free block
            auto pv = std::prev(nx);
            if (pv->first + pv->second == o) {
                o = pv->first;
                sz += pv->second;
                free_.erase(pv);
            }
        }
        free_[o] = sz;
    }
    size_t capacity() const { return cap_; }
    size_t used() {
        std::lock_guard<std::mutex> lk(mu_);
        return used_;
    }
    size_t largest_free() {
        std::lock_guard<std::mutex> lk(mu_);
        size_t m = 0;
        for (auto& f : free_) m = f.second > m ? f.second : m;
        return m;
    }

   private:
    char* base_ = nullptr;
    size_t cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_, taken_;
    std::mutex mu_;
};

}  // namespace qp
