// Host-side launchers for the state-vector kernels (implemented in
// kernels.cu). All launches are asynchronous on the given stream; functions
// returning a value read it back with a synchronous copy on that stream.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "hqs_desc.h"

namespace hqs {

// Reduction scratch: per-CTA partial sums (device) plus a pinned host slot.
struct ReduceScratch {
    double* d_partials = nullptr;  // kMaxPartials * 4 doubles
    double* d_result = nullptr;    // 4 doubles
    double* h_result = nullptr;    // pinned, 4 doubles
};
constexpr int kMaxPartials = 2048;

int device_sm_count();

// One fused pass over the state (see hqs_desc.h). mats: device pool of the
// pass's matrices in the arithmetic's element format. Returns a cudaError_t.
cudaError_t launch_pass(int arith, void* state, const void* mats, const PassDesc& d, cudaStream_t s);
size_t pass_smem_bytes(int arith, const PassDesc& d);
// Resident CTAs per SM the pass kernel for (arith, d) is compiled for (its
// register budget); shared memory may allow fewer.
int pass_reg_ctas(int arith, const PassDesc& d);

// Tensor-memory pass over a complex128 state (umma_pass.cu): the pass's
// element-wise matrices (double-float, at the start of mats) and the dense
// gate's digit block (at u.gate_off). The TMA tensor map is built from the
// descriptor and the state pointer.
cudaError_t launch_umma_pass(void* state, const void* mats, const UmmaDesc& u, cudaStream_t s);
size_t umma_smem_bytes();
// Whether a tensor-memory pass on the current device ran out of a bounded
// wait since the last call (the error word is cleared).
cudaError_t umma_check_error(bool* failed);

// One entry of a batched launch: a pass over one state. Device-resident.
struct BatchItem {
    void* state;
    const void* mats;      // device pointer to the pass's matrix pool
    uint64_t tile_begin;   // first global tile index of this item
    PassDesc desc;
};
// Run every item's pass in one launch (total_tiles = sum of the items' tiles,
// smem = the largest pass_smem_bytes of the items). With arith == kArithTC,
// tc selects the tensor-core kernel (needed when any item has TC gates).
cudaError_t launch_batch(int arith, bool tc, const BatchItem* d_items, int nitems, uint64_t total_tiles, size_t smem,
                         cudaStream_t s);

// Sum of |a_i|^2 over indices with (i & mask) == val.
cudaError_t reduce_probability(int arith, const void* state, int n, uint64_t mask, uint64_t val,
                               ReduceScratch& rs, cudaStream_t s, double* out);
// P(bit pos = 0) and P(bit pos = 1) in one sweep.
cudaError_t reduce_bit_probs(int arith, const void* state, int n, int pos, ReduceScratch& rs,
                             cudaStream_t s, double* out2);
// -sum p log2 p.
cudaError_t reduce_entropy(int arith, const void* state, int n, ReduceScratch& rs, cudaStream_t s,
                           double* out);
// nblocks partial sums of |a|^2 over contiguous blocks, written to d_out (device).
cudaError_t block_sums(int arith, const void* state, int n, uint64_t nblocks, double* d_out, cudaStream_t s);
// Pauli-sum expectation: sum_t Re(c_t <psi|P_t|psi>); masks/coefs in device memory.
// With zonly (one term, no X or Y) the device masks are not read: out is the
// signed norm sum_i (-1)^popcount(i & zmask0) |a_i|^2, to be scaled by Re(c).
// E[t] = sum_i (-1)^popcount(i & z[t]) |a_i|^2 for T <= 64 masks (device
// array d_z) in one read of the state; d_scratch holds
// zparity_multi_scratch_bytes(T); out (host, T doubles) receives E. Synchronizes s.
cudaError_t reduce_zparity_multi(int arith, const void* state, int n, int T, const uint64_t* d_z, double* d_scratch,
                                 cudaStream_t s, double* out);
size_t zparity_multi_scratch_bytes(int T);
cudaError_t reduce_pauli_expectation(int arith, const void* state, int n, int nterms, const uint64_t* d_xm,
                                     const uint64_t* d_ym, const uint64_t* d_zm, const double* d_coef,
                                     ReduceScratch& rs, cudaStream_t s, double* out, bool zonly = false,
                                     uint64_t zmask0 = 0);

// out = sum_t c_t P_t in (out-of-place; out and in must not alias). d_coef: per
// term the pair (c_t i^{|Y_t|}, -c_t i^{|Y_t|}) in the arithmetic's matrix format.
cudaError_t pauli_apply(int arith, const void* in, void* out, int n, int nterms, const uint64_t* d_xm,
                        const uint64_t* d_ym, const uint64_t* d_zm, const double* d_coef, cudaStream_t s);
// Zero amplitudes with (i & mask) != val, scale the others by scale.
cudaError_t collapse_scale(int arith, void* state, int n, uint64_t mask, uint64_t val, double scale,
                           cudaStream_t s);
// Every amplitude := value.
cudaError_t fill_value(int arith, void* state, uint64_t count, double re, double im, cudaStream_t s);
// Remove bit pos from the index keeping the half where it equals keep (in place).
cudaError_t drop_bit(int arith, void* state, int n, int pos, int keep, cudaStream_t s);
// In-place bit permutation: new state bit newpos[j] takes old bit oldpos[j]
// (j < m); all other bits stay. {oldpos} and {newpos} are the same set.
cudaError_t permute_bits(int arith, void* state, int n, int m, const uint8_t* oldpos, const uint8_t* newpos,
                         cudaStream_t s);
// complex64 <-> complex128 conversions for host transfers (c64 storage).
cudaError_t c64_to_c128(const void* in, void* out, uint64_t count, cudaStream_t s);
cudaError_t c128_to_c64(const void* in, void* out, uint64_t count, cudaStream_t s);

}  // namespace hqs
