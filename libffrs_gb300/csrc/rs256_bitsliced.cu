// Bitsliced RS256 kernels (filled in by the fast-path implementation).
#include "common.cuh"
#include "rs256.cuh"

namespace ffgpu {

bool rs256_fast_init(Rs256Code &) { return false; }
void rs256_fast_free(Rs256Code &) {}
bool rs256_fast_encode(const Rs256Code &, const uint8_t *, size_t, int, uint8_t *, cudaStream_t) { return false; }
bool rs256_fast_decode(const Rs256Code &, uint8_t *, uint8_t *, size_t, int, uint8_t *, cudaStream_t) { return false; }

}  // namespace ffgpu
