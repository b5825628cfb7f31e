// Host engine behind the _cppsim_mpi.SimulatorMPI drop-in: one state vector
// resident in the HBM of one GB300, driven by the kernels of kernels.cu.
//
// Semantics follow src/simulator-mpi/SimulatorMPI.{hpp,cpp} on one rank (no
// global qubits): qubit ids map to state-bit positions (locals_), gates are
// fused in FP64 on the host with the reference's rules, run() applies the
// fused gate, queries see the state as of the last run(). Execution is
// deferred: run() appends the fused gate to a pending list that is planned
// into multi-gate passes (one HBM sweep each) and launched asynchronously; any
// call that observes or reshapes the state flushes the list first.
#pragma once
#include <cuda_runtime.h>

#include <chrono>
#include <complex>
#include <cstdint>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "fusion.h"
#include "hqs_desc.h"
#include "hqs_kernels.h"
#include "workspace.h"

namespace hqs {

enum Precision : int { kC128 = 0, kC64 = 1 };

struct PauliTerm {
    std::vector<std::pair<int64_t, char>> ops;  // (index into ids, 'X'|'Y'|'Z')
    cplx coef;
};

struct EngineStats {
    uint64_t gates = 0;          // apply_controlled_gate calls
    uint64_t runs = 0;           // run() calls that produced a fused gate
    uint64_t passes = 0;         // state sweeps launched by the apply planner
    uint64_t pass_ops = 0;       // fused gates applied by those sweeps
    uint64_t bytes_moved = 0;    // algorithmic HBM bytes of the apply sweeps
    uint64_t flushes = 0;
};

class Engine {
public:
    Engine(uint64_t seed, int64_t max_local, int64_t max_cluster_size, int precision, int arith);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // --- reference API (SimulatorMPI.hpp:63-225) ---
    void allocate_qubit(int64_t id);
    void allocate_qureg(const std::vector<int64_t>& ids, cplx init);
    void deallocate_qubit(int64_t id);
    void apply_controlled_gate(const std::vector<cplx>& m, int dim, const std::vector<int64_t>& ids,
                               const std::vector<int64_t>& ctrls);
    void run();
    std::vector<bool> measure_qubits(const std::vector<int64_t>& ids);
    double get_probability(const std::vector<bool>& bits, const std::vector<int64_t>& ids);
    cplx get_amplitude(const std::vector<bool>& bits, const std::vector<int64_t>& ids);
    void collapse_wavefunction(const std::vector<int64_t>& ids, const std::vector<bool>& values);
    double entropy();
    std::vector<int64_t> get_qubits_ids() const { return locals_; }
    std::vector<int64_t> get_local_qubits_ids() const { return locals_; }
    std::vector<int64_t> get_global_qubits_ids() const { return {}; }
    void set_qubits_perm(const std::vector<int64_t>& p);
    void swap_qubits(const std::vector<int64_t>& pairs);
    // state in position order (2^n complex128 values)
    void cheat_local(cplx* out, size_t cap);
    // --- methods the Python backend calls that the reference never bound ---
    double get_expectation_value(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids);
    // One value per operator (extension): the distinct Z strings of the
    // operators made only of Z strings share one read of the state per 64;
    // the other operators go through get_expectation_value.
    std::vector<double> get_expectation_values(const std::vector<std::vector<PauliTerm>>& ops,
                                               const std::vector<int64_t>& ids);
    void apply_qubit_operator(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids);
    void set_wavefunction(const cplx* wf, size_t len, const std::vector<int64_t>& ids);

    // --- extras ---
    size_t num_qubits() const { return locals_.size(); }
    int precision() const { return precision_; }
    int arith() const { return arith_; }
    void synchronize();
    void flush();  // launch every pending fused gate
    const EngineStats& stats() const { return stats_; }
    // Sampled full-register outcomes: one uniform draw per shot from the
    // engine's RNG, no collapse. out[s] = basis index (position order).
    void sample(uint64_t shots, uint64_t* out);
    // Move the qubits ids to the given state positions with one in-place
    // permutation sweep (the ids previously at those positions take the
    // vacated ones).
    void move_qubits(const std::vector<int64_t>& ids, const std::vector<int>& positions);
    // Fused-pass planner knobs.
    void set_pass_limits(int max_tile_bits, int max_ops, int defer);
    void* device_state() { return state_; }
    Workspace& workspace() { return ws_; }
    cudaStream_t stream() const { return ws_.stream(); }

private:
    [[noreturn]] void fail(const std::string& msg) const { throw std::runtime_error(msg); }
    size_t find_sure(int64_t id) const;   // throws the reference's ArrayFindSure message
    long find(int64_t id) const;
    void ensure_capacity(uint64_t amps);
    void grow_one();
    void masks_for(const std::vector<int64_t>& ids, const std::vector<bool>& bits, uint64_t& msk,
                   uint64_t& val) const;
    double probability_internal(uint64_t msk, uint64_t val);
    void normalize(double norm, uint64_t msk, uint64_t val);
    void pauli_masks(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids,
                     std::vector<uint64_t>& xm, std::vector<uint64_t>& ym, std::vector<uint64_t>& zm) const;
    uint64_t sample_index(double rnd, bool& ok, double* total);
    uint64_t scan_block(uint64_t i, uint64_t K, double rnd) const;
    size_t elem_bytes() const { return precision_ == kC64 ? 8 : 16; }
    int n() const { return (int)locals_.size(); }

    int precision_, arith_;
    int64_t min_local_, max_local_, max_cluster_;
    std::vector<int64_t> locals_;
    Fusion fused_;
    std::mt19937 rnd_eng_;
    std::uniform_real_distribution<double> dist_{0.0, 1.0};

    Workspace ws_;
    void* state_ = nullptr;          // device
    void* spare_ = nullptr;          // second state buffer for apply_qubit_operator
    uint64_t spare_cap_ = 0;
    uint64_t capacity_ = 0;          // amplitudes
    double* block_dev_ = nullptr;    // up to 2^15 block sums
    double* block_host_ = nullptr;   // pinned
    cplx* scan_host_ = nullptr;      // pinned copy of one measurement block
    size_t scan_cap_ = 0;

    std::vector<GateOp> pending_;
    int max_tile_bits_ = 11;
    int max_ops_ = 16;
    int defer_ = 64;                 // launch when this many fused gates are pending
    EngineStats stats_;
};

}  // namespace hqs
