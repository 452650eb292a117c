// Host-logic check of the decode planner's parallel build (test
// infrastructure): the frames given on the command line, repeated to at
// least 600, are planned serially and on 4 threads; the two plans and their
// device layouts (task descriptors with fake, widely separated base
// addresses) must be equal byte for byte.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "dec_plan.h"
using namespace ozl;

int main(int argc, char** argv)
{
    std::vector<std::vector<uint8_t>> files;
    for (int i = 1; i < argc; i++) {
        std::ifstream f(argv[i], std::ios::binary);
        files.emplace_back((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    }
    if (files.empty()) return 2;
    std::vector<const uint8_t*> hp;
    std::vector<size_t> fs;
    while (hp.size() < 600)
        for (auto& v : files) {
            hp.push_back(v.data());
            fs.push_back(v.size());
        }
    size_t const n = hp.size();
    DecodePlan a, b;
    std::string ea, eb;
    int ra = a.build(n, hp.data(), fs.data(), nullptr, true, true, ea);
    int rb = b.buildParallel(n, hp.data(), fs.data(), nullptr, true, true, eb, 4);
    if (ra || rb) {
        printf("plan errors %d %d %s %s\n", ra, rb, ea.c_str(), eb.c_str());
        return 1;
    }
    int bad = 0;
    auto eq = [&](bool c, const char* what) {
        if (!c) {
            printf("DIFF %s\n", what);
            bad++;
        }
    };
    eq(a.frames.size() == b.frames.size(), "frames");
    eq(a.streams.size() == b.streams.size(), "streams");
    eq(a.nodes.size() == b.nodes.size(), "nodes");
    eq(a.hashes.size() == b.hashes.size(), "hashes");
    eq(a.arenaBytes == b.arenaBytes, "arena");
    eq(a.totalOut == b.totalOut, "totalOut");
    eq(a.params == b.params, "params");
    std::vector<const uint8_t*> dF(n);
    std::vector<uint8_t*> dO(n);
    uint64_t out = 0;
    for (size_t i = 0; i < n; i++) {
        dF[i] = reinterpret_cast<const uint8_t*>(0x100000000ull + i * 0x1000000ull);
        dO[i] = reinterpret_cast<uint8_t*>(0x900000000000ull + out);
        out += (a.frames[i].decodedSize + 255) & ~uint64_t(255);
    }
    uint8_t* const dA = reinterpret_cast<uint8_t*>(0x300000000000ull);
    uint8_t* const dP = reinterpret_cast<uint8_t*>(0x400000000000ull);
    uint8_t* const dS = reinterpret_cast<uint8_t*>(0x500000000000ull);
    uint8_t* const dPool = reinterpret_cast<uint8_t*>(0x600000000000ull);
    DeviceLayout la, lb;
    std::string e1, e2;
    int r1 = layoutPlan(a, dF.data(), dO.data(), dA, dP, dS, dPool, la, e1);
    int r2 = layoutPlan(b, dF.data(), dO.data(), dA, dP, dS, dPool, lb, e2);
    eq(r1 == 0 && r2 == 0, "layout status");
    eq(la.pool == lb.pool, "descriptor pool bytes");
    eq(la.scratchBytes == lb.scratchBytes, "scratch");
    eq(la.launches.size() == lb.launches.size(), "launch count");
    for (size_t i = 0; i < la.launches.size() && i < lb.launches.size(); i++) {
        const Launch& x = la.launches[i];
        const Launch& y = lb.launches[i];
        eq(x.kind == y.kind && x.level == y.level && x.taskOff == y.taskOff && x.nbTasks == y.nbTasks
               && x.tileOff == y.tileOff && x.nbTiles == y.nbTiles && x.param0 == y.param0 && x.algoBytes == y.algoBytes,
           "launch");
    }
    printf("frames=%zu nodes=%zu streams=%zu launches=%zu pool=%zu bad=%d\n", n, a.nodes.size(), a.streams.size(),
           la.launches.size(), la.pool.size(), bad);
    return bad ? 1 : 0;
}
