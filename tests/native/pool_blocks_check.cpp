// Serving pool allocator (ozl::PoolBlocks) against a byte-map model: random
// take/give sequences over a small range. After every step the free blocks
// are disjoint, sorted, merged (no two touch), inside the range, and cover
// exactly the bytes the model holds free; take() returns the lowest offset
// whose free run holds the request, and fails only when no run does;
// largest() is the longest free run. Prints "bad=0" when every check held.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "pool_blocks.h"

int main(int argc, char** argv)
{
    unsigned const seed = argc > 1 ? unsigned(std::atoi(argv[1])) : 1u;
    std::mt19937_64 rng(seed);
    long bad = 0, takes = 0, fails = 0;
    for (int round = 0; round < 200; round++) {
        size_t const range = 1 + rng() % 4096;
        ozl::PoolBlocks p;
        p.reset(range);
        std::vector<char> used(range, 0);
        std::vector<std::pair<size_t, size_t>> live;
        for (int step = 0; step < 400; step++) {
            bool const doTake = live.empty() || rng() % 3 != 0;
            if (doTake) {
                size_t const want = 1 + rng() % (1 + range / (1 + rng() % 8));
                // model: the first free run, in offset order, of at least `want` bytes
                size_t expect = range;
                for (size_t o = 0; o < range && expect == range;) {
                    if (used[o]) { o++; continue; }
                    size_t e = o;
                    while (e < range && !used[e]) e++;
                    if (e - o >= want) expect = o;
                    o = e;
                }
                size_t off = 0;
                bool const ok = p.take(want, off);
                if (ok != (expect < range)) bad++;
                if (ok) {
                    takes++;
                    if (off != expect) bad++;
                    for (size_t b = off; b < off + want && b < range; b++) {
                        if (used[b]) bad++;
                        used[b] = 1;
                    }
                    live.emplace_back(off, want);
                } else {
                    fails++;
                }
            } else {
                size_t const k = rng() % live.size();
                auto const blk = live[k];
                live.erase(live.begin() + long(k));
                p.give(blk.first, blk.second);
                for (size_t b = blk.first; b < blk.first + blk.second; b++) used[b] = 0;
            }
            // invariants
            size_t prevEnd = 0, freeBytes = 0, longest = 0;
            bool first = true;
            for (auto& f : p.free) {
                if (f.second == 0 || f.first + f.second > range) bad++;
                if (!first && f.first <= prevEnd) bad++; // sorted, disjoint and not touching
                for (size_t b = f.first; b < f.first + f.second && b < range; b++)
                    if (used[b]) bad++;
                prevEnd = f.first + f.second;
                freeBytes += f.second;
                longest = f.second > longest ? f.second : longest;
                first = false;
            }
            size_t modelFree = 0, run = 0, modelLongest = 0;
            for (size_t b = 0; b < range; b++) {
                modelFree += used[b] ? 0 : 1;
                run = used[b] ? 0 : run + 1;
                modelLongest = run > modelLongest ? run : modelLongest;
            }
            if (freeBytes != modelFree || p.largest() != longest || longest != modelLongest) bad++;
        }
    }
    std::printf("takes=%ld fails=%ld bad=%ld\n", takes, fails, bad);
    return bad ? 1 : 0;
}
