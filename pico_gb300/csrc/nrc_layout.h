// Layout shared by the host and the device code of the neural radiance cache:
// sizes, the swizzled operand layout and the hash-grid geometry.
//
// Operand layout.  Every matrix the network multiplies is a stack of rows of
// 64 bf16 values (128 bytes), grouped in 1024-byte atoms of 8 rows with the
// 128-byte swizzle: element (row r, column c) of a tile whose base is
// 1024-byte aligned sits at
//     (r / 8) * 1024 + (r % 8) * 128 + (((c / 8) ^ (r % 8)) * 16) + (c % 8) * 2.
// The same bytes serve as a K-major operand (K = the 64 columns: activations
// times weights in the forward pass) and as an MN-major operand (K = the rows:
// the weight gradient dW = dY^T X sums over the batch rows, and the input
// gradient dX = dY W reads the weights with K = their output rows), so nothing
// is ever transposed.  Both descriptor byte offsets are 1024: the stride
// between 8-row groups along K (MN-major) or along M/N (K-major).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pico {
namespace nrc {

constexpr int kLevels = 16;          // hash-grid levels, 2 features each
constexpr int kWidth = 64;           // network width and padded input width
constexpr int kRows = 128;           // rows per tile = TMEM lanes = MMA M
constexpr int kHidden = 5;           // 64 x 64 layers; layer 5 maps 64 -> 16 (3 used)
constexpr int kLayers = 6;
constexpr int kOutRows = 16;         // padded output width (MMA N)
constexpr int kOutputs = 3;
constexpr uint32_t kTileBytes = kRows * kWidth * 2;          // 16384
constexpr uint32_t kLayerBytes = kWidth * kWidth * 2;        // 8192
constexpr uint32_t kOutBytes = kOutRows * kWidth * 2;        // 2048
constexpr uint32_t kWeightBytes = kHidden * kLayerBytes + kOutBytes;   // 43008
constexpr uint32_t kWeightRegion = 44032;                    // kWeightBytes rounded up to 1024
constexpr uint32_t kGuardBytes = 2048;                       // garbage rows of M = 128 weight-gradient MMAs
constexpr int kInputHash = 0, kInputSH = 32, kInputNormal = 48, kInputRough = 51, kInputAlbedo = 52,
              kInputBias = 55;

// Byte offset of the 16-byte chunk `chunk` (columns 8*chunk .. 8*chunk+7) of row `row`.
__host__ __device__ __forceinline__ uint32_t swz(uint32_t row, uint32_t chunk)
{
    return (row >> 3) * 1024u + (row & 7u) * 128u + ((chunk ^ (row & 7u)) << 4);
}

// Byte offset of parameter (layer, out row, in column) in the swizzled bf16 weight image.
__host__ __device__ __forceinline__ uint32_t weight_offset(uint32_t layer, uint32_t o, uint32_t i)
{
    return layer * kLayerBytes + swz(o, i >> 3) + (i & 7u) * 2u;
}

// Hash-grid geometry: per level the scale of the unit cube and, for dense
// levels, the grid points per axis; hashed levels use the spatial hash of
// Mueller et al. 2022 (primes 1, 2654435761, 805459861) modulo the table size.
struct GridGeometry {
    float scale[kLevels];
    uint32_t res1[kLevels];          // points per axis of a dense level, 0 for hashed levels
    uint32_t table_mask;             // entries per level - 1 (a power of two)
    uint32_t log2_table;
    float lo[3], inv_extent[3];      // position normalisation to the unit cube
};

}  // namespace nrc
}  // namespace pico
