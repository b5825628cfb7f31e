// Per-simulator device resources: a CUDA stream, the matrix pool and its
// pinned staging buffer, reduction scratch, and the fused-pass planner that
// turns a list of fused gates into sweeps over the state.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "hqs_desc.h"
#include "hqs_kernels.h"

namespace hqs {

using cplx = std::complex<double>;

// One fused gate in state positions.
struct GateOp {
    int k = 0;                 // 0..5 targets (0 = scalar factor)
    bool diag = false;
    int pos[kMaxK] = {0, 0, 0, 0, 0};  // state position of matrix bit j
    uint64_t ctrl_mask = 0;    // state positions that must be 1
    std::vector<cplx> m;       // dense: dim*dim row-major; diag: dim entries; k == 0: 1 entry
    // tensor-core pool bytes of this gate, computed once when the gate is
    // reused across many flushes (the batched server); empty: computed on use
    std::shared_ptr<const std::vector<unsigned char>> tc_pool;
};

struct PassPlan {
    PassDesc desc;
    size_t pool_off = 0;       // byte offset of the pass's matrices in the pool
    uint64_t bytes = 0;        // algorithmic HBM bytes of the sweep
};

class CudaError : public std::runtime_error {
public:
    explicit CudaError(const std::string& m) : std::runtime_error(m) {}
};

void cuda_check(cudaError_t e, const char* what);

class Workspace {
public:
    Workspace();
    ~Workspace();
    Workspace(const Workspace&) = delete;
    Workspace& operator=(const Workspace&) = delete;

    cudaStream_t stream() const { return stream_; }
    // Wait for the stream, then fail (CudaError) if a tensor-memory pass on
    // this device ran out of one of its bounded waits since the last check.
    void synchronize_checked();
    ReduceScratch& reduce() { return rs_; }
    // Device scratch of at least `bytes` (grown on demand; contents undefined).
    void* scratch(size_t bytes);
    // Plan the ops into passes (max_tile_bits, max_ops per pass) and launch
    // them on the stream. Returns the algorithmic bytes moved.
    uint64_t apply_ops(void* state, int n, int arith, const std::vector<GateOp>& ops, int max_tile_bits,
                       int max_ops, uint64_t* passes_out = nullptr);
    // Upload `bytes` from host memory into a device buffer owned by the
    // workspace (reused between calls; valid until the next upload).
    void* upload(const void* host, size_t bytes);

    static size_t mat_elem_bytes(int arith) { return arith_is_c64(arith) ? 8 : 16; }

    // Per-launch device timing of the apply passes (CUDA events around each
    // launch on the workspace stream). collect_timing() waits for the events,
    // returns the totals since the last collection and clears them.
    struct LaunchRecord {
        int kind = 0;  // 0: pass kernel, 1: tensor-memory pass
        int nops = 0;  // gate ops the launch applies
        int copies = 0;  // tensor-memory pass: TMA copies per tile
        uint64_t target_mask = 0;  // tensor-memory pass: the dense gate's five (padded) target positions
        uint64_t bytes = 0;
        double ms = 0.0;
    };
    struct PassTiming {
        uint64_t launches = 0;
        uint64_t bytes = 0;
        double ms = 0.0;
        std::vector<LaunchRecord> log;  // one record per launch, in launch order
    };
    void set_timing(bool on) { timing_ = on; }
    PassTiming collect_timing();

private:
    void ensure_pool(size_t bytes);
    void ensure_pinned(size_t bytes);

    cudaStream_t stream_ = nullptr;
    ReduceScratch rs_;
    void* pool_ = nullptr;
    size_t pool_bytes_ = 0;
    void* pinned_ = nullptr;
    size_t pinned_bytes_ = 0;
    cudaEvent_t staging_free_ = nullptr;
    bool staging_pending_ = false;
    void* scratch_ = nullptr;
    size_t scratch_bytes_ = 0;
    void* up_ = nullptr;
    size_t up_bytes_ = 0;
    bool timing_ = false;
    struct TimedLaunch {
        cudaEvent_t a, b;
        uint64_t bytes;
        int kind, nops, copies;
        uint64_t target_mask;
    };
    std::vector<TimedLaunch> timed_;
    std::vector<cudaEvent_t> event_pool_;
    cudaEvent_t take_event();
};

// One launch of apply_ops: a tiled pass of the pass kernel, or a
// tensor-memory pass (one dense gate on the tcgen05 tensor cores with the
// diagonal / scalar gates around it, complex128 tensor-core arithmetic).
struct LaunchPlan {
    bool umma = false;
    PassPlan pass;          // tiled pass (pass.pool_off unused)
    UmmaDesc udesc;         // tensor-memory pass
    size_t first = 0;       // index of the launch's first op
    size_t pool_off = 0;    // byte offset of the launch's matrices in the pool
    size_t pool_bytes = 0;
    uint64_t bytes = 0;     // algorithmic HBM bytes of the sweep
};
// Whether apply_ops may use tensor-memory passes (HQS_UMMA=0 turns them off).
bool umma_enabled();
// Whether a gate can be the dense gate of a tensor-memory pass.
bool umma_candidate(int arith, const GateOp& op);
// The launches apply_ops makes for ops: tensor-memory passes around every
// candidate dense gate (when allowed and n >= 12), the pass planner for the
// rest.
std::vector<LaunchPlan> plan_launches(int n, int arith, const std::vector<GateOp>& ops, int max_tile_bits, int max_ops,
                                      bool allow_umma);
// Matrices of a tensor-memory pass (ops: the pass's gates, in order).
void write_umma_pool(const UmmaDesc& u, const GateOp* ops, unsigned char* dst);

// Bytes of a planned pass's matrix pool and the pool itself (ops are the
// pass's gates, in order), in the arithmetic's element format.
size_t pass_pool_bytes(int arith, const PassDesc& d);
void write_pass_pool(int arith, const PassDesc& d, const GateOp* ops, unsigned char* dst);

// Build the pass descriptors for ops (exposed for host-side tests of the planner).
// min_ctas: trailing ops that would bring the pass below this many resident
// CTAs per SM (or below its first op's, if fewer) start the next pass; -1
// keeps the first op's occupancy (the right trade when a sweep is
// expensive), 0 never leaves ops out (batched serving of small states, bound
// by host work per pass).
std::vector<PassPlan> plan_passes(int n, int arith, const GateOp* ops, size_t nops, int max_tile_bits, int max_ops,
                                  std::vector<size_t>* op_first = nullptr, size_t max_passes = SIZE_MAX,
                                  int min_ctas = -1);
inline std::vector<PassPlan> plan_passes(int n, int arith, const std::vector<GateOp>& ops, int max_tile_bits,
                                         int max_ops, std::vector<size_t>* op_first = nullptr) {
    return plan_passes(n, arith, ops.data(), ops.size(), max_tile_bits, max_ops, op_first);
}
// Whether the planner runs this gate on the tensor cores (when the tile
// allows), and the tensor-core pool bytes of such a gate, for GateOp::tc_pool.
bool tc_candidate(int arith, const GateOp& op);
std::shared_ptr<const std::vector<unsigned char>> make_tc_pool(int arith, const GateOp& op);

}  // namespace hqs
