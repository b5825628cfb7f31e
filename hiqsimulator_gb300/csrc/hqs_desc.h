// Descriptors shared by the host engine and the CUDA kernels.
//
// A "pass" streams the whole state vector once through shared memory in
// tiles. A tile is the set of 2^q amplitudes whose indices agree on every
// state bit outside tile_pos[0..q); tile-local index bit j is state bit
// tile_pos[j] (ascending, so tile_pos[0..w) == 0..w-1 is the contiguous run
// that makes global loads coalesced). Every op of the pass acts only on tile
// bits, so applying the op list tile by tile equals applying each op to the
// whole state in order.
#pragma once
#include <stdint.h>

namespace hqs {

constexpr int kMaxOpsPerPass = 24;
constexpr int kMaxTileBits = 12;
constexpr int kMaxK = 5;
constexpr uint8_t kOuterSlot = 0x80;

// Arithmetic used by the apply kernels.
enum Arith : int32_t {
    kArithF64 = 1,  // complex128 storage, native FP64 arithmetic
    kArithDF = 2,   // complex128 storage, double-float (2 x FP32) arithmetic, ~48-bit
    kArithF32 = 3,  // complex64 storage, FP32 arithmetic
    kArithTC = 4,   // complex128 storage, dense 3..5-qubit gates on the fp16 tensor cores
                    // (exact digit products, see apply_tc), the rest in double-float
    kArithTF32 = 5, // complex64 storage, dense 3..5-qubit gates as 3xTF32 tensor-core
                    // products (see apply_tf32), the rest in FP32
    kArithTC64 = 6, // complex64 storage, dense 3..5-qubit gates as exact two-digit fp16
                    // products (apply_tc), the rest in FP32
};

// complex64 (float2) states
constexpr bool arith_is_c64(int a) { return a == kArithF32 || a == kArithTF32 || a == kArithTC64; }
// arithmetic whose pool carries tensor-core gates
constexpr bool arith_has_tc(int a) { return a == kArithTC || a == kArithTF32 || a == kArithTC64; }

// Tensor-core digit planes: every real operand is written as kTcDigits signed
// base-2^10 digits (|d| <= 512) scaled by a power of two shared by its row.
constexpr int kTcDigits = 5;
// complex64 states use two such digits per state real and three per gate real
constexpr int kTcDigits64 = 2;
constexpr int kTcDigits64B = 3;

struct OpDesc {
    int32_t k;            // targets (0 = scalar multiply of the whole tile)
    int32_t diag;         // 1: matrix pool holds only the 2^k diagonal entries
    uint32_t ctrl_local;  // tile-local bits that must all be 1
    uint32_t mat_off;     // offset (elements) of this op's matrix in the pass pool
    uint64_t ctrl_outer;  // state bits outside the tile that must all be 1
    uint8_t tslot[kMaxK]; // tile-local bit of matrix bit j; diagonal gates may have targets
                          // outside the tile: kOuterSlot | state position
    uint8_t tc;           // 1: dense gate applied on the tensor cores (digit planes in the pool)
    uint8_t pad[2];
};

struct PassDesc {
    int32_t n;            // state qubits
    int32_t q;            // tile bits
    int32_t w;            // contiguous low run: tile_pos[j] == j for j < w
    int32_t nops;
    int32_t nins;         // number of sorted positions in ins_pos
    uint32_t mat_elems;   // pool elements staged into shared memory
    uint32_t tc_bytes;    // shared-memory scratch for tensor-core digit planes (0: none)
    uint32_t prefetch;    // 1: each CTA copies its next tile into a staging buffer while it
                          //    computes the current one (cp.async); 2: every op works in place,
                          //    the next tile streams into the second tile buffer
    uint64_t fixed_mask;  // state bits forced to 1 for every processed tile
    uint8_t tile_pos[kMaxTileBits];
    uint8_t ins_pos[64];  // sorted union of tile_pos and fixed-mask positions
    OpDesc ops[kMaxOpsPerPass];
};

// Tensor-memory pass (complex128): one dense gate on the tcgen05 tensor cores
// plus runs of diagonal / scalar gates before and after it, over tiles of
// 2^12 amplitudes: five target positions (gates on fewer qubits are widened
// with identity factors) and 128 index groups, the MMA's M. Every real is
// written as six balanced base-2^9 digits; the tile's tensor-memory
// accumulators hold the six digit levels of each output.
constexpr int kUmmaTileBits = 12;
constexpr int kUmmaGroups = 128;
constexpr int kUmmaDigits = 6;
constexpr uint32_t kUmmaGatePlaneBytes = 6 * 64 * 128;           // six gate digit planes, 64 rows x 128 B
constexpr uint32_t kUmmaGateBytes = kUmmaGatePlaneBytes + 64 * 4;  // + column exponents
// complex64: four gate digit planes, then the column exponents
constexpr uint32_t kUmmaGatePlaneBytes64 = 4 * 64 * 128;
constexpr uint32_t kUmmaGateBytes64 = kUmmaGatePlaneBytes64 + 64 * 4;
constexpr uint32_t kUmmaEwMaxBytes = 13 * 512;                     // element-wise matrices staged per pass
constexpr int kUmmaRunBits = 8;                                    // tile bits a diagonal run's factor may depend on

struct UmmaDesc {
    PassDesc d;            // tile (q = 12), fixed mask, ops; ops[tc_op] is the dense gate
    int32_t tc_op;
    uint32_t gate_off;     // byte offset of the gate block in the pool (1024-aligned)
    uint32_t ew_bytes;     // bytes of element-wise matrices at the start of the pool
    uint32_t box_bytes;    // bytes of one TMA box; a tile is 2^nextra boxes
    uint8_t tslot[5];      // tile slots of the five targets, ascending (element bits 0..4)
    uint8_t rank;          // tensor-map rank (1..5)
    uint8_t nextra;        // tile bits above the box (one copy per combination)
    uint8_t c64;           // 1: complex64 state (three digits per state real, four per gate real), 0: complex128
    int8_t dim_kind[5];    // 1: a run of tile positions (the box) and the gap above it (coordinate
                           // from the tile base); 2: the same, last, with the extra tile bits above
                           // its run (coordinate from the tile base plus the copy's extra bits)
    int8_t dim_pos[5];     // first state position of each dimension
    int8_t dim_bits[5];    // state positions each dimension spans
    int8_t dim_box[5];     // of them, the run of tile positions at the bottom (inside the box)
    int8_t extra_pos[kMaxTileBits];  // state positions of the extra tile bits, ascending
    uint32_t run_mask[2];  // tile slots the element-wise run before (0) / after (1) the dense gate
                           // depends on (targets and controls inside the tile), at most kUmmaRunBits
};

// true when any op of the pass runs on the tensor cores
inline bool pass_has_tc(const PassDesc& d) {
    for (int o = 0; o < d.nops; ++o)
        if (d.ops[o].tc) return true;
    return false;
}

}  // namespace hqs
