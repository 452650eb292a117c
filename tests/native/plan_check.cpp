#include <map>
// Host-logic check of the decode planner (test infrastructure): builds the
// plan and layout of a frame with fake, widely separated base addresses and
// verifies that every pointer and length a task uses lies inside an allocation.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>
#include <string>
#include "dec_plan.h"
using namespace ozl;
struct Range { const char* name; uintptr_t lo, hi; };
std::vector<Range> R;
bool gQuiet = false;
#define LOG(...) do { if (!gQuiet) printf(__VA_ARGS__); } while (0)
bool inR(const void* p, uint64_t len, const char* what) {
  uintptr_t a = (uintptr_t)p;
  for (auto& r : R) if (a >= r.lo && a + len <= r.hi) return true;
  printf("BAD %s ptr=%lx len=%lu\n", what, (unsigned long)a, (unsigned long)len);
  return false;
}
// 0: planned, every task in bounds; 1: a task out of bounds; 2: the planner
// or the layout refused the frame
static int checkFrame(const std::vector<uint8_t>& fr) {
  DecodePlan plan; std::string err;
  const uint8_t* hp = fr.data(); size_t fs = fr.size();
  int rc = plan.build(1, &hp, &fs, nullptr, true, true, err);
  if (rc) { LOG("plan err %d %s\n", rc, err.c_str()); return 2; }
  uint8_t* dF = (uint8_t*)0x100000000ull; uint8_t* dO = (uint8_t*)0x200000000ull;
  uint8_t* dA = (uint8_t*)0x300000000ull; uint8_t* dP = (uint8_t*)0x400000000ull;
  uint8_t* dS = (uint8_t*)0x500000000ull; uint8_t* dPool = (uint8_t*)0x600000000ull;
  const uint8_t* dFs[1] = {dF}; uint8_t* dOs[1] = {dO};
  DeviceLayout L;
  rc = layoutPlan(plan, dFs, dOs, dA, dP, dS, dPool, L, err);
  if (rc) { LOG("layout err %d %s\n", rc, err.c_str()); return 2; }
  R = {{"frame",(uintptr_t)dF,(uintptr_t)dF+fs},{"out",(uintptr_t)dO,(uintptr_t)dO+plan.totalOut},
       {"arena",(uintptr_t)dA,(uintptr_t)dA+plan.arenaBytes},{"params",(uintptr_t)dP,(uintptr_t)dP+plan.params.size()},
       {"scratch",(uintptr_t)dS,(uintptr_t)dS+L.scratchBytes},{"pool",(uintptr_t)dPool,(uintptr_t)dPool+L.pool.size()}};
  LOG("out=%lu arena=%lu params=%zu scratch=%lu pool=%zu launches=%zu\n", (unsigned long)plan.totalOut,
    (unsigned long)plan.arenaBytes, plan.params.size(), (unsigned long)L.scratchBytes, L.pool.size(), L.launches.size());
  int bad = 0;
  auto P = [&](size_t off) { return L.pool.data() + off; };
  auto hostPtrs = [&](const uint8_t* const* dp, int n, std::vector<const uint8_t*>& v) {
    size_t off = (const uint8_t*)dp - dPool; memcpy(v.data(), L.pool.data() + off, n * sizeof(void*)); };
  std::map<const uint64_t*, std::pair<const uint8_t*, uint32_t>> fusedSums;
  for (auto& l : L.launches) {
    LOG(" launch kind=%d level=%d tasks=%u tiles=%u\n", l.kind, l.level, l.nbTasks, l.nbTiles);
    for (uint32_t i = 0; i < l.nbTasks; i++) {
      switch (l.kind) {
        case KIND_CONST: { auto t = ((ConstTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.n*t.w, "const.out"); bad += !inR(t.value, t.w, "const.val"); break; }
        case KIND_COPY: { auto t = ((CopyTask*)P(l.taskOff))[i];
          bad += !inR(t.dst, t.bytes, "copy.dst"); bad += !inR(t.src, t.bytes, "copy.src"); break; }
        case KIND_FSE: { auto t = ((FseTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.dstSize, "fse.out"); bad += !inR(t.bits, t.bitsSize, "fse.bits");
          bad += !inR(t.norm, 2*t.nbSym, "fse.norm"); break; }
        case KIND_HUF: { auto t = ((HufTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.dstSize, "huf.out"); bad += !inR(t.bits, t.bitsSize, "huf.bits");
          bad += !inR(t.weights, t.nbWeights, "huf.w"); break; }
        case KIND_NUMPIPE: { auto t = ((NumPipeTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.n*t.w, "np.out");
          uint64_t ns = t.delta ? t.n-1 : t.n;
          if (t.srcMode == SRC_PLAIN) bad += !inR(t.src, ns*t.w, "np.src");
          else if (t.srcMode == SRC_BITPACK) bad += !inR(t.src, (ns*t.nbBits+7)/8, "np.bits");
          else { bad += !inR(t.planes, t.w*8, "np.planes"); std::vector<const uint8_t*> v(t.w); hostPtrs(t.planes, t.w, v);
                 for (auto p : v) bad += !inR(p, ns, "np.plane"); }
          if (t.blockSums) {  // fused content-checksum block sums: whole blocks of this output
            bad += !inR(t.blockSums, (uint64_t)t.hashBlocks*64, "np.sums");
            if ((uint64_t)t.hashBlocks * 1024 > t.n * t.w) { printf("BAD np.hashBlocks beyond the output\n"); bad++; }
            fusedSums[t.blockSums] = std::make_pair(t.out, t.hashBlocks);
          }
          LOG("   np n=%lu w=%u mode=%u zz=%u delta=%u nbBits=%u tileBase=%u fused=%u\n",(unsigned long)t.n,t.w,t.srcMode,t.zigzag,t.delta,t.nbBits,t.tileBase,t.hashBlocks);
          break; }
        case KIND_HASH: { auto t = ((HashTask*)P(l.taskOff))[i];
          bad += !inR(t.data, t.len, "hash.data"); if (t.nbBlocks) bad += !inR(t.blockSums, t.nbBlocks*64, "hash.sums");
          // every full block's sums come from exactly one producer: the hash
          // launch's own block list, or the numeric task writing this output
          uint32_t listed = 0;
          const TileRef* tl = (const TileRef*)P(l.tileOff);
          for (uint32_t k = 0; k < l.nbTiles; k++) listed += tl[k].task == i;
          auto f = fusedSums.find(t.blockSums);
          bool const fused = t.nbBlocks && f != fusedSums.end();
          if (fused && (listed || f->second.first != t.data || f->second.second != t.nbBlocks)) {
            printf("BAD hash %u: fused sums do not match the task\n", i); bad++; }
          if (!fused && listed != t.nbBlocks) { printf("BAD hash %u: %u of %u blocks listed\n", i, listed, t.nbBlocks); bad++; }
          break; }
        case KIND_TOKENIZE: { auto t = ((TokenizeTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.n*t.w, "tok.out"); bad += !inR(t.idx, t.n*t.iw, "tok.idx"); bad += !inR(t.alphabet, (uint64_t)t.alphabetSize*t.w, "tok.alpha"); break; }
        case KIND_WIDEN: { auto t = ((WidenTask*)P(l.taskOff))[i];
          bad += !inR(t.src, t.n*t.w, "widen.src"); bad += !inR(t.dst, t.n*4, "widen.dst"); break; }
        case KIND_FLOATDEC: { auto t = ((FloatDecTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.n*(t.eltType?2:4), "flt.out"); bad += !inR(t.exponent, t.n, "flt.ex"); break; }
        case KIND_FLATPACK: { auto t = ((FlatpackTask*)P(l.taskOff))[i];
          bad += !inR(t.out, t.n, "flat.out"); break; }
        default: break;
      }
    }
    if (l.nbTiles) bad += !inR(P(l.tileOff) - L.pool.data() + dPool, l.nbTiles * 8, "tiles");
    if (l.needsScan) bad += !inR(dS + l.statusOff, l.statusBytes, "scan");
  }
  LOG("bad=%d\n", bad);
  return bad != 0;
}

// plan_check FRAME: the frame's plan, printed, and its bounds check.
// plan_check FRAME --fuzz N SEED: N mutated copies of the frame (bytes
// flipped, set to 0x00 or 0xFF, or the frame truncated), each either refused
// by the planner or planned with every task in bounds.
int main(int argc, char** argv) {
  std::ifstream f(argv[1], std::ios::binary);
  std::vector<uint8_t> fr((std::istreambuf_iterator<char>(f)), {});
  if (argc < 5 || strcmp(argv[2], "--fuzz") != 0) {
    int const r = checkFrame(fr);
    if (r == 2) return 1;
    return r;
  }
  gQuiet = true;
  long const n = atol(argv[3]);
  uint64_t s = (uint64_t)atoll(argv[4]) * 0x9E3779B97F4A7C15ull + 1;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  long planned = 0, refused = 0, bad = 0;
  for (long k = 0; k < n && !fr.empty(); k++) {
    std::vector<uint8_t> m = fr;
    int const kinds = 1 + (int)(rnd() % 3);
    for (int q = 0; q < kinds; q++) {
      // half the mutations in the first 96 bytes, where the frame and block headers are
      size_t const lim = (rnd() & 1) ? std::min<size_t>(m.size(), 96) : m.size();
      if (m.empty()) break;
      size_t const at = rnd() % lim;
      switch (rnd() % 4) {
        case 0: m[at] ^= (uint8_t)(1u << (rnd() % 8)); break;
        case 1: m[at] ^= (uint8_t)(1 + rnd() % 255); break;
        case 2: m[at] = (rnd() & 1) ? 0x00 : 0xFF; break;
        default: m.resize(at); break;
      }
    }
    int const r = checkFrame(m);
    if (r == 0) planned++; else if (r == 2) refused++; else bad++;
  }
  printf("fuzz planned=%ld refused=%ld bad=%ld\n", planned, refused, bad);
  return bad != 0;
}
