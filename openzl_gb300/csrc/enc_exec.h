// Launchers of the encode kernels (encode_kernels.cu).
#pragma once
#include <cuda_runtime.h>

#include "enc_tasks.h"

namespace ozl {

cudaError_t prepareEncodeKernels();
uint32_t hufEncStreamCap(uint32_t segmentSize);
void launchEncMax(const EncNumTask* t, const TileRef* tiles, uint32_t nbTiles, unsigned long long* maxima,
                  cudaStream_t s);
void launchEncNum(const EncNumTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
void launchPack(const PackTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
void launchHist(const HistTask* t, uint32_t n, uint32_t* hists, cudaStream_t s);
// FSE normalization, header and encoding table of each chunk; a failed
// normalization sets errors[0].
void launchFseTables(const FseTableTask* t, uint32_t n, uint32_t* sizes, uint32_t* errors, cudaStream_t s);
void launchFseEnc(const FseEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s);
// chunks with a fields scratch (four states, kFseLongMin symbols or more)
void launchFseEncLong(const FseEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s);
// Huffman code lengths, codes and weights of each chunk.
void launchHufTables(const HufTableTask* t, uint32_t n, cudaStream_t s);
void launchHufEnc(const HufEncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s);
void launchPut(const PutTask* t, uint32_t n, cudaStream_t s);
void launchBf16(const Bf16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
// Tokenize, up to the per-task distinct counts (counts[task], errors[0]).
void launchTokCount(const TokTask* t, uint32_t nbTasks, const TileRef* tiles, uint32_t nbTiles, uint64_t* tileSums,
                    uint64_t* tilePrefix, uint32_t* counts, uint32_t* errors, cudaStream_t s);
// 16-bit chunks: value counts, first occurrences and maxima.
void launchHist16(const Hist16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
// 16-bit chunks: tokenize indices.
void launchTok16(const Tok16Task* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
// 16-bit-symbol Huffman streams, one thread per stream.
void launchHuf16Enc(const Huf16EncTask* t, uint32_t n, uint32_t* sizes, cudaStream_t s);
// Sorted tokenize: indices renumbered to the sorted alphabet.
void launchRemap(const RemapTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);
// Tokenize, the alphabet and the indices (iw set in the tasks).
void launchTokEmit(const TokTask* t, const TileRef* tiles, uint32_t nbTiles, cudaStream_t s);

} // namespace ozl
