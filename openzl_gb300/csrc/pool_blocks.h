// First-fit allocator of a byte range: the serving loop's shared HBM pool
// (host bookkeeping only; the server calls it under its lock). Free blocks
// are kept by offset and merged with their neighbours when returned.
#pragma once
#include <cstddef>
#include <iterator>
#include <map>

namespace ozl {

struct PoolBlocks {
    std::map<size_t, size_t> free; // offset -> bytes
    void reset(size_t bytes)
    {
        free.clear();
        if (bytes) free.emplace(0, bytes);
    }
    size_t largest() const
    {
        size_t m = 0;
        for (auto& f : free) m = f.second > m ? f.second : m;
        return m;
    }
    // the lowest free block that holds `bytes` gives its first `bytes`
    bool take(size_t bytes, size_t& off)
    {
        for (auto it = free.begin(); it != free.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            size_t const rest = it->second - bytes;
            free.erase(it);
            if (rest) free.emplace(off + bytes, rest);
            return true;
        }
        return false;
    }
    // returns a block that take() gave
    void give(size_t off, size_t bytes)
    {
        auto it = free.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free.erase(nx);
        }
        if (it != free.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free.erase(it);
            }
        }
    }
};

} // namespace ozl
