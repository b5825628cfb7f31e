// Batched circuit server: many independent small circuits resident in HBM at
// once, advanced together.
//
// A request is a circuit on n qubits (qubit ids 0..n-1 at positions 0..n-1)
// plus what to return: the amplitude of |0...0>, one full-register sample for
// a given uniform draw, or the expectation of a Pauli-string sum. Requests
// wait in arrival order until their state (2^n amplitudes) fits the HBM byte
// budget and a slot is free; then their state is allocated with the
// stream-ordered allocator and set to |0...0>. Every round builds, for each
// resident circuit that still has gates, the next tiled pass of its fused
// gates (the same planner as the single-state engine) and runs all of them in
// one batched launch, so circuits admitted while others are in flight share
// the GPU. A circuit whose last pass has been launched is finished in the
// next round, after that round's launches: its result is computed on a second
// stream that waits only for the round that ran its last pass (so the host
// reads results while the GPU runs the next round), then its memory is
// released, which admits waiting requests. Results do not depend on which
// other circuits share a round.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <exception>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fusion.h"
#include "hqs_kernels.h"
#include "workspace.h"

namespace hqs {

enum ResultKind : int { kResultAmplitude0 = 0, kResultSample = 1, kResultExpectation = 2 };

struct ServerGate {
    std::vector<cplx> m;            // dim x dim row-major
    std::vector<int> targets;       // qubit indices (matrix bit j <-> targets[j])
    std::vector<int> ctrls;
};

struct ServerResult {
    uint64_t id;
    int kind;
    double value_re, value_im;      // amplitude, or expectation in value_re
    uint64_t sample;                // basis index for kResultSample
    double submit_s, admit_s, done_s;  // host clock (seconds) at each stage
    uint32_t passes;                // fused passes the circuit took
};

// Serving complex128 states of this many qubits or more run their dense
// gates as tensor-memory launches (one per state per round; 64 or more tiles
// of 4096 amplitudes); smaller states stay in the batched tiled launches.
constexpr int kServeUmmaBits = 18;

class Server {
public:
    Server(int precision, int arith, uint64_t budget_bytes, int max_active, int cluster_size);
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    // Checks the gates and queues the request; worker threads fuse them on
    // the host (consecutive gates while their qubits fit in cluster_size) and
    // precompute the tensor-core pools while earlier requests run, and the
    // request is admitted, in arrival order, once that is done. pauli_*
    // describe the Pauli sum for kResultExpectation (x/y/z masks over qubit
    // indices, complex coefs).
    uint64_t submit(int n, const std::vector<ServerGate>& gates, int kind, double rnd,
                    const std::vector<uint64_t>& pauli_x, const std::vector<uint64_t>& pauli_y,
                    const std::vector<uint64_t>& pauli_z, const std::vector<cplx>& pauli_coef);
    // One round: finish, admit, plan, launch. Returns results that completed.
    std::vector<ServerResult> step();
    // Run rounds until nothing is queued or resident.
    std::vector<ServerResult> drain();
    size_t queued() const { return queue_.size(); }
    size_t active() const { return active_.size(); }
    uint64_t bytes_in_use() const { return bytes_in_use_; }
    uint64_t rounds() const { return rounds_; }
    uint64_t launches() const { return launches_; }
    // host seconds in step(): batching, staging waits, launches, results,
    // admissions, total
    void timing(double out[6]) const {
        for (int i = 0; i < 6; ++i) out[i] = t_phase_[i];
        out[0] -= t_phase_[1] + t_phase_[2];
    }
    cudaStream_t stream() const { return ws_.stream(); }

private:
    // Host preparation of one request, filled by a worker thread: the fused
    // gates planned into passes, and every pass's matrices already in the
    // kernels' format in one host pool (pass k at plans[k].pool_off).
    struct Prep {
        int n = 0;
        std::vector<ServerGate> gates;
        std::vector<PassPlan> plans;
        std::vector<uint8_t> plan_tc;      // pass runs tensor-core gates
        std::vector<uint32_t> plan_smem;   // shared-memory bytes of the pass
        // tensor-memory launches (complex128 states of kServeUmmaBits qubits
        // or more): the launch's descriptor and pool bytes (its pool at
        // plans[k].pool_off)
        std::vector<uint8_t> plan_umma;
        std::vector<UmmaDesc> plan_udesc;
        std::vector<uint32_t> plan_pool;
        std::vector<unsigned char> pool;
        std::exception_ptr error;
        std::atomic<bool> ready{false};
    };
    struct Req {
        uint64_t id;
        int n;
        int kind;
        double rnd;
        std::shared_ptr<Prep> prep;  // the request's passes; next = first pass not yet launched
        size_t next = 0;
        std::vector<uint64_t> px, py, pz;
        std::vector<cplx> pc;
        void* state = nullptr;
        uint64_t bytes = 0;
        double submit_s = 0, admit_s = 0;
        uint32_t passes = 0;
    };
    ServerResult finish(Req& r);
    double now() const;
    double t_phase_[6] = {0, 0, 0, 0, 0, 0};
    void prepare(Prep& p) const;
    void worker();

    int precision_, arith_, max_active_, cluster_;
    uint64_t budget_, bytes_in_use_ = 0;
    uint64_t next_id_ = 1, rounds_ = 0, launches_ = 0;
    std::deque<Req> queue_;
    std::vector<Req> active_;
    Workspace ws_;   // rounds: planning uploads, batched launches, admissions
    Workspace wsr_;  // results of finished circuits
    cudaEvent_t step_done_ = nullptr;  // end of the previous step (its round and admissions)
    cudaEvent_t freed_ = nullptr;      // after the last frees on the results stream
    void* staging_[2] = {nullptr, nullptr};  // pinned: items + matrices
    size_t staging_bytes_[2] = {0, 0};
    cudaEvent_t staging_done_[2] = {nullptr, nullptr};
    void* dev_[2] = {nullptr, nullptr};
    size_t dev_bytes_[2] = {0, 0};
    int flip_ = 0;
    double* blocks_dev_ = nullptr;
    double* blocks_host_ = nullptr;
    std::vector<std::complex<double>> scan_;
    double t0_;
    // preparation workers: FIFO jobs, at most kPrepAhead prepared requests
    // waiting for admission
    static constexpr size_t kPrepAhead = 256;
    std::mutex mu_;
    std::condition_variable cv_work_, cv_ready_;
    std::deque<std::shared_ptr<Prep>> jobs_;
    size_t prepared_waiting_ = 0;
    bool stop_ = false;
    std::vector<std::thread> workers_;
};

}  // namespace hqs
