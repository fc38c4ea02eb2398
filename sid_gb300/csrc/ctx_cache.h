// ctx_cache.h -- small per-CUDA-context cache of values resolved once per
// context (plain C++, no CUDA types, so that the key logic is testable on a
// host without a GPU).
//
// A device address taken from a module (cudaGetSymbolAddress) belongs to the
// context that loaded the module.  After cudaDeviceReset, or with a second
// driver context on the same device, the same device ordinal has a new context
// and the old address is stale.  Keys are therefore the driver's unique
// context IDs (cuCtxGetId: never reused within a process), not device ordinals.
#pragma once
#include <cstddef>
#include <mutex>
#include <utility>
#include <vector>

namespace sid {

template <class T>
class CtxCache {
public:
    // Value for context `id`; on a miss `resolve(T*)` is called (returning 0
    // on success) and its value kept.  A failed resolve is not cached.
    template <class Resolve>
    int get(unsigned long long id, Resolve&& resolve, T* out)
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (const auto& e : entries_)
            if (e.first == id) {
                *out = e.second;
                return 0;
            }
        T v{};
        const int rc = resolve(&v);
        if (rc != 0) return rc;
        entries_.emplace_back(id, v);
        *out = v;
        return 0;
    }
    size_t size() const
    {
        std::lock_guard<std::mutex> lk(mu_);
        return entries_.size();
    }

private:
    mutable std::mutex mu_;
    std::vector<std::pair<unsigned long long, T>> entries_;
};

}  // namespace sid
