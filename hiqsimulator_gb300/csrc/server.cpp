#include "server.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <stdexcept>

namespace hqs {

namespace {

// A fused gate (DenseGate over ids 0..n-1, ids == positions) as a GateOp, the
// way SimulatorMPI::Run dispatches it (SimulatorMPI.cpp:470-524).
bool to_gate_op(const DenseGate& g, const std::vector<int64_t>& ctrls, GateOp& op) {
    op = GateOp();
    op.k = (int)g.ids.size();
    if (op.k > kMaxK) throw std::runtime_error("server: a fused gate acts on more than 5 qubits");
    if (op.k == 0) {
        if (g.m[0] == cplx(1.0, 0.0)) return false;
        op.m = {g.m[0]};
        return true;
    }
    for (int j = 0; j < op.k; ++j) op.pos[j] = (int)g.ids[j];
    for (int64_t c : ctrls) op.ctrl_mask |= 1ULL << c;
    op.diag = g.diag;
    if (g.diag) {
        op.m.resize(g.dim);
        for (int r = 0; r < g.dim; ++r) op.m[r] = g.m[(size_t)r * g.dim + r];
    } else {
        op.m = g.m;
    }
    return true;
}

}  // namespace

Server::Server(int precision, int arith, uint64_t budget_bytes, int max_active, int cluster_size)
    : precision_(precision),
      arith_(arith),
      max_active_(std::max(1, max_active)),
      cluster_(std::max(1, std::min(cluster_size, kMaxK))),
      budget_(budget_bytes) {
    if (arith_ == 0) arith_ = precision_ == 1 ? kArithTC64 : kArithTC;
    if (precision_ == 1 && arith_ == kArithTC) arith_ = kArithTC64;
    if ((precision_ == 1) != arith_is_c64(arith_)) throw std::invalid_argument("server: precision/arith mismatch");
    for (int i = 0; i < 2; ++i)
        cuda_check(cudaEventCreateWithFlags(&staging_done_[i], cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventCreateWithFlags(&step_done_, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventRecord(step_done_, ws_.stream()), "cudaEventRecord");
    cuda_check(cudaEventCreateWithFlags(&freed_, cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaMalloc(&blocks_dev_, sizeof(double) << 15), "cudaMalloc(blocks)");
    cuda_check(cudaMallocHost(&blocks_host_, sizeof(double) << 15), "cudaMallocHost(blocks)");
    t0_ = 0;
    t0_ = now();
    const unsigned hw = std::thread::hardware_concurrency();
    const unsigned nw = std::max(1u, std::min(8u, hw > 1 ? hw - 1 : 1u));
    for (unsigned i = 0; i < nw; ++i) workers_.emplace_back(&Server::worker, this);
}

Server::~Server() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    for (auto& t : workers_) t.join();
    cudaStreamSynchronize(wsr_.stream());
    cudaStreamSynchronize(ws_.stream());
    for (auto& r : active_)
        if (r.state) cudaFreeAsync(r.state, ws_.stream());
    cudaStreamSynchronize(ws_.stream());
    for (int i = 0; i < 2; ++i) {
        cudaFreeHost(staging_[i]);
        cudaFree(dev_[i]);
        cudaEventDestroy(staging_done_[i]);
    }
    cudaEventDestroy(step_done_);
    cudaEventDestroy(freed_);
    cudaFree(blocks_dev_);
    cudaFreeHost(blocks_host_);
}

double Server::now() const {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count() - t0_;
}

uint64_t Server::submit(int n, const std::vector<ServerGate>& gates, int kind, double rnd,
                        const std::vector<uint64_t>& pauli_x, const std::vector<uint64_t>& pauli_y,
                        const std::vector<uint64_t>& pauli_z, const std::vector<cplx>& pauli_coef) {
    if (n < 1 || n > 40) throw std::invalid_argument("server: qubit count out of range");
    for (const auto& sg : gates) {
        const int dim = 1 << sg.targets.size();
        if ((size_t)dim * dim != sg.m.size()) throw std::invalid_argument("server: matrix size does not match targets");
        if ((int)sg.targets.size() > kMaxK) throw std::invalid_argument("server: a gate acts on more than 5 qubits");
        for (int t : sg.targets)
            if (t < 0 || t >= n) throw std::invalid_argument("server: target out of range");
        for (int c : sg.ctrls)
            if (c < 0 || c >= n) throw std::invalid_argument("server: control out of range");
    }
    Req r;
    r.id = next_id_++;
    r.n = n;
    r.kind = kind;
    r.rnd = rnd;
    r.px = pauli_x;
    r.py = pauli_y;
    r.pz = pauli_z;
    r.pc = pauli_coef;
    r.bytes = ((uint64_t)1 << n) * (precision_ == 1 ? 8 : 16);
    r.submit_s = now();
    r.prep = std::make_shared<Prep>();
    r.prep->n = n;
    r.prep->gates = gates;
    {
        std::lock_guard<std::mutex> lk(mu_);
        jobs_.push_back(r.prep);
    }
    cv_work_.notify_one();
    queue_.push_back(std::move(r));
    return queue_.back().id;
}

// Sequential greedy fusion: gates join the current fused gate while the union
// of their qubits stays within cluster_; controlled gates too large to fuse go
// alone with their controls as a control mask. Then the passes and their
// matrix pools.
void Server::prepare(Prep& p) const {
    Fusion fu;
    uint64_t cur = 0;
    std::vector<GateOp> ops;
    auto flush = [&]() {
        if (fu.empty()) return;
        DenseGate g;
        std::vector<int64_t> ctrls;
        fu.perform(g, ctrls);
        GateOp op;
        if (to_gate_op(g, ctrls, op)) ops.push_back(std::move(op));
        fu.clear();
        cur = 0;
    };
    for (const auto& sg : p.gates) {
        const int dim = 1 << sg.targets.size();
        uint64_t q = 0;
        for (int t : sg.targets) q |= 1ULL << t;
        for (int c : sg.ctrls) q |= 1ULL << c;
        DenseGate g;
        g.dim = dim;
        g.m = sg.m;
        g.diag = is_diagonal(sg.m, dim);
        g.ids.assign(sg.targets.begin(), sg.targets.end());
        std::vector<int64_t> cs(sg.ctrls.begin(), sg.ctrls.end());
        if ((int)(sg.targets.size() + sg.ctrls.size()) > cluster_) {
            flush();
            fu.insert(std::move(g), cs);
            flush();
            continue;
        }
        if (__builtin_popcountll(cur | q) > cluster_) flush();
        add_controls(g, cs);
        fu.insert(std::move(g), {});
        cur |= q;
    }
    flush();
    p.gates.clear();
    p.gates.shrink_to_fit();
    // plan every pass: small states take tiles up to 2^12 amplitudes (the
    // planner shrinks them to fit shared memory) and up to 24 gates, so a
    // circuit needs few rounds. complex128 tensor-core passes keep their first
    // gate's occupancy: their digit scratch grows with the tile, and a batched
    // launch runs at its largest item's (measured: 109 circuits/s against 104
    // at a floor of 2 CTAs per SM and 86 with no floor)
    // complex128 states of kServeUmmaBits qubits or more: every dense
    // 3-5-qubit gate as a tensor-memory launch of its own (with the diagonal
    // runs around it), the other gates in batched tiled passes. complex64
    // states stay batched: their two-digit tiled passes are cheap enough that
    // one launch per state costs more (measured: 179 against 281 circuits/s)
    if (arith_ == kArithTC && p.n >= kServeUmmaBits && umma_enabled()) {
        std::vector<LaunchPlan> L = plan_launches(p.n, arith_, ops, kMaxTileBits, kMaxOpsPerPass, true);
        size_t total = 0;
        for (auto& l : L) {
            total = (total + 1023) & ~(size_t)1023;
            l.pool_off = total;
            total += (l.pool_bytes + 255) & ~(size_t)255;
        }
        p.pool.assign(std::max<size_t>(total, 256), 0);
        const size_t K = L.size();
        p.plans.resize(K);
        p.plan_tc.assign(K, 0);
        p.plan_smem.assign(K, 0);
        p.plan_umma.assign(K, 0);
        p.plan_udesc.resize(K);
        p.plan_pool.assign(K, 0);
        for (size_t k = 0; k < K; ++k) {
            p.plan_pool[k] = (uint32_t)L[k].pool_bytes;
            if (L[k].umma) {
                p.plan_umma[k] = 1;
                p.plan_udesc[k] = L[k].udesc;
                p.plans[k].pool_off = L[k].pool_off;
                write_umma_pool(L[k].udesc, ops.data() + L[k].first, p.pool.data() + L[k].pool_off);
                continue;
            }
            p.plans[k] = L[k].pass;
            p.plans[k].pool_off = L[k].pool_off;
            PassDesc& d = p.plans[k].desc;
            d.prefetch = 0;  // the batched kernel loads its tiles directly
            write_pass_pool(arith_, d, ops.data() + L[k].first, p.pool.data() + L[k].pool_off);
            p.plan_tc[k] = pass_has_tc(d) ? 1 : 0;
            p.plan_smem[k] = (uint32_t)pass_smem_bytes(arith_, d);
        }
        return;
    }
    std::vector<size_t> first;
    p.plans = plan_passes(p.n, arith_, ops.data(), ops.size(), kMaxTileBits, kMaxOpsPerPass, &first, SIZE_MAX,
                          arith_ == kArithTC ? -1 : 0);
    size_t total = 256;
    for (const auto& pl : p.plans) total = std::max(total, pl.pool_off + pass_pool_bytes(arith_, pl.desc));
    p.pool.assign(total, 0);
    p.plan_tc.resize(p.plans.size());
    p.plan_smem.resize(p.plans.size());
    p.plan_umma.assign(p.plans.size(), 0);
    for (size_t k = 0; k < p.plans.size(); ++k) {
        PassDesc& d = p.plans[k].desc;
        d.prefetch = 0;  // the batched kernel loads its tiles directly
        write_pass_pool(arith_, d, ops.data() + first[k], p.pool.data() + p.plans[k].pool_off);
        p.plan_tc[k] = pass_has_tc(d) ? 1 : 0;
        p.plan_smem[k] = (uint32_t)pass_smem_bytes(arith_, d);
    }
}

void Server::worker() {
    for (;;) {
        std::shared_ptr<Prep> job;
        {
            std::unique_lock<std::mutex> lk(mu_);
            cv_work_.wait(lk, [&] { return stop_ || (!jobs_.empty() && prepared_waiting_ < kPrepAhead); });
            if (stop_) return;
            job = jobs_.front();
            jobs_.pop_front();
        }
        try {
            prepare(*job);
        } catch (...) {
            job->error = std::current_exception();
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            job->ready.store(true, std::memory_order_release);
            ++prepared_waiting_;
        }
        cv_ready_.notify_all();
    }
}

ServerResult Server::finish(Req& r) {
    ServerResult res{};
    res.id = r.id;
    res.kind = r.kind;
    res.submit_s = r.submit_s;
    res.admit_s = r.admit_s;
    res.passes = r.passes;
    cudaStream_t s = wsr_.stream();
    const size_t eb = precision_ == 1 ? 8 : 16;
    if (r.kind == kResultAmplitude0) {
        if (eb == 8) {
            float v[2];
            cuda_check(cudaMemcpyAsync(v, r.state, 8, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            res.value_re = v[0];
            res.value_im = v[1];
        } else {
            double v[2];
            cuda_check(cudaMemcpyAsync(v, r.state, 16, cudaMemcpyDeviceToHost, s), "cudaMemcpyAsync");
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            res.value_re = v[0];
            res.value_im = v[1];
        }
    } else if (r.kind == kResultSample) {
        const uint64_t N = 1ULL << r.n;
        const uint64_t nb = std::min<uint64_t>(N, 1ULL << 15);
        cuda_check(block_sums(arith_, r.state, r.n, nb, blocks_dev_, s), "block_sums");
        cuda_check(cudaMemcpyAsync(blocks_host_, blocks_dev_, nb * sizeof(double), cudaMemcpyDeviceToHost, s),
                   "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        std::partial_sum(blocks_host_, blocks_host_ + nb, blocks_host_);
        uint64_t i = std::lower_bound(blocks_host_, blocks_host_ + nb, r.rnd) - blocks_host_;
        if (i == nb) i = nb - 1;
        const uint64_t K = N / nb;
        scan_.resize(K);
        if (eb == 8) {
            std::vector<float> tmp(2 * K);
            cuda_check(cudaMemcpyAsync(tmp.data(), static_cast<unsigned char*>(r.state) + i * K * 8, K * 8,
                                       cudaMemcpyDeviceToHost, s),
                       "cudaMemcpyAsync");
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            for (uint64_t j = 0; j < K; ++j) scan_[j] = cplx(tmp[2 * j], tmp[2 * j + 1]);
        } else {
            cuda_check(cudaMemcpyAsync(scan_.data(), static_cast<unsigned char*>(r.state) + i * K * 16, K * 16,
                                       cudaMemcpyDeviceToHost, s),
                       "cudaMemcpyAsync");
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
        double shift = i > 0 ? blocks_host_[i - 1] : 0.0;
        uint64_t k = i * K;
        for (uint64_t j = 0; j < K; ++j, ++k) {
            shift += std::norm(scan_[j]);
            if (shift >= r.rnd) break;
        }
        res.sample = std::min(k, N - 1);
    } else {
        const size_t T = r.px.size();
        std::vector<unsigned char> blob(T * (3 * 8 + 16) + 16);
        std::memcpy(blob.data(), r.px.data(), T * 8);
        std::memcpy(blob.data() + T * 8, r.py.data(), T * 8);
        std::memcpy(blob.data() + 2 * T * 8, r.pz.data(), T * 8);
        double* co = reinterpret_cast<double*>(blob.data() + 3 * T * 8);
        for (size_t t = 0; t < T; ++t) {
            co[2 * t] = r.pc[t].real();
            co[2 * t + 1] = r.pc[t].imag();
        }
        double out = 0.0;
        if (T > 0) {
            const unsigned char* d = static_cast<const unsigned char*>(wsr_.upload(blob.data(), blob.size()));
            cuda_check(reduce_pauli_expectation(arith_, r.state, r.n, (int)T, (const uint64_t*)d,
                                                (const uint64_t*)(d + T * 8), (const uint64_t*)(d + 2 * T * 8),
                                                (const double*)(d + 3 * T * 8), wsr_.reduce(), s, &out),
                       "reduce_pauli_expectation");
        }
        res.value_re = out;
    }
    bool failed = false;  // a tensor-memory launch's bounded wait ran out
    cuda_check(umma_check_error(&failed), "umma_check_error");
    if (failed) throw CudaError("tensor-memory pass: a bounded device wait ran out (results of the pass are invalid)");
    cuda_check(cudaFreeAsync(r.state, s), "cudaFreeAsync");
    r.state = nullptr;
    bytes_in_use_ -= r.bytes;
    res.done_s = now();
    return res;
}

std::vector<ServerResult> Server::step() {
    const double t_start = now();
    std::vector<ServerResult> done;
    cudaStream_t s = ws_.stream();
    // circuits whose last pass ran in an earlier round finish after this
    // round's launches, overlapping them
    std::vector<size_t> finishing;
    for (size_t i = 0; i < active_.size(); ++i)
        if (active_[i].next >= active_[i].prep->plans.size()) finishing.push_back(i);
    if (!queue_.empty() && active_.empty() && queue_.front().bytes > budget_)
        throw std::runtime_error("server: a request needs more HBM than the admission budget");
    // 1. the next pass of every resident circuit (planned at preparation)
    struct Planned {
        Req* r;
        size_t k;
        bool tc;
        size_t smem;
    };
    std::vector<Planned> planned, umma;
    for (auto& r : active_) {
        if (r.next >= r.prep->plans.size()) continue;
        const Planned pl{&r, r.next, r.prep->plan_tc[r.next] != 0, r.prep->plan_smem[r.next]};
        if (r.prep->plan_umma[r.next]) umma.push_back(pl);
        else planned.push_back(pl);
        ++r.next;
        ++r.passes;
    }
    // 2. one launch per (kernel, shared-memory class): a launch runs at the
    // occupancy of its largest pass, so passes are grouped by footprint
    auto smem_class = [](size_t b) { return b <= 56 * 1024 ? 0 : b <= 75 * 1024 ? 1 : b <= 112 * 1024 ? 2 : 3; };
    std::stable_sort(planned.begin(), planned.end(), [&](const Planned& a, const Planned& b) {
        if (a.tc != b.tc) return a.tc > b.tc;
        return smem_class(a.smem) < smem_class(b.smem);
    });
    // one of the two pinned staging buffers and its device copy, at least
    // total bytes, once the copy that last used it has finished
    auto staging = [&](size_t total, unsigned char*& host, unsigned char*& dev) {
        const int f = flip_;
        flip_ ^= 1;
        const double tw = now();
        cuda_check(cudaEventSynchronize(staging_done_[f]), "cudaEventSynchronize");
        t_phase_[1] += now() - tw;
        if (staging_bytes_[f] < total) {
            cudaFreeHost(staging_[f]);
            staging_[f] = nullptr;
            staging_bytes_[f] = 0;
            cuda_check(cudaMallocHost(&staging_[f], total * 2), "cudaMallocHost(staging)");
            staging_bytes_[f] = total * 2;
        }
        if (dev_bytes_[f] < total) {
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
            cudaFree(dev_[f]);
            dev_[f] = nullptr;
            dev_bytes_[f] = 0;
            cuda_check(cudaMalloc(&dev_[f], total * 2), "cudaMalloc(batch)");
            dev_bytes_[f] = total * 2;
        }
        host = static_cast<unsigned char*>(staging_[f]);
        dev = static_cast<unsigned char*>(dev_[f]);
        return f;
    };
    // tensor-memory launches: one per large state, pools staged together
    if (!umma.empty()) {
        size_t total = 0;
        for (const auto& u : umma) total += (u.r->prep->plan_pool[u.k] + 1023) & ~(size_t)1023;
        unsigned char *host = nullptr, *dev = nullptr;
        const int f = staging(total, host, dev);
        size_t off = 0;
        const double tl = now();
        for (const auto& u : umma) {
            std::memcpy(host + off, u.r->prep->pool.data() + u.r->prep->plans[u.k].pool_off, u.r->prep->plan_pool[u.k]);
            off += (u.r->prep->plan_pool[u.k] + 1023) & ~(size_t)1023;
        }
        cuda_check(cudaMemcpyAsync(dev, host, total, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(umma)");
        cuda_check(cudaEventRecord(staging_done_[f], s), "cudaEventRecord");
        off = 0;
        for (const auto& u : umma) {
            cuda_check(launch_umma_pass(u.r->state, dev + off, u.r->prep->plan_udesc[u.k], s), "launch_umma_pass");
            off += (u.r->prep->plan_pool[u.k] + 1023) & ~(size_t)1023;
            ++launches_;
        }
        t_phase_[2] += now() - tl;
    }
    auto launch = [&](size_t lo, size_t hi) {
        const bool tc = planned[lo].tc;
        const size_t nitems = hi - lo;
        const size_t head = ((nitems * sizeof(BatchItem)) + 255) & ~(size_t)255;
        size_t total = head;
        for (size_t i = lo; i < hi; ++i)
            total += pass_pool_bytes(arith_, planned[i].r->prep->plans[planned[i].k].desc);
        unsigned char *host = nullptr, *dev = nullptr;
        const int f = staging(total, host, dev);
        BatchItem* bi = reinterpret_cast<BatchItem*>(host);
        size_t off = head;
        uint64_t tiles = 0;
        size_t smem = 0;
        for (size_t i = lo; i < hi; ++i) {
            const PassPlan& pl = planned[i].r->prep->plans[planned[i].k];
            const PassDesc& d = pl.desc;
            BatchItem& b = bi[i - lo];
            b.state = planned[i].r->state;
            b.mats = dev + off;
            b.tile_begin = tiles;
            b.desc = d;
            std::memcpy(host + off, planned[i].r->prep->pool.data() + pl.pool_off, pass_pool_bytes(arith_, d));
            off += pass_pool_bytes(arith_, d);
            tiles += 1ULL << (d.n - d.nins);
            smem = std::max(smem, planned[i].smem);
        }
        const double tl = now();
        cuda_check(cudaMemcpyAsync(dev, host, total, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(batch)");
        cuda_check(cudaEventRecord(staging_done_[f], s), "cudaEventRecord");
        cuda_check(launch_batch(arith_, tc, reinterpret_cast<const BatchItem*>(dev), (int)nitems, tiles, smem, s),
                   "launch_batch");
        t_phase_[2] += now() - tl;
        ++launches_;
    };
    for (size_t lo = 0; lo < planned.size();) {
        size_t hi = lo + 1;
        while (hi < planned.size() && planned[hi].tc == planned[lo].tc &&
               smem_class(planned[hi].smem) == smem_class(planned[lo].smem))
            ++hi;
        launch(lo, hi);
        lo = hi;
    }
    ++rounds_;
    const double t_res = now();
    t_phase_[0] += t_res - t_start;  // batching, waits and launches (split below)
    // 3. results of the circuits collected above: the results stream waits
    // for the end of the previous step (the round that ran their last passes
    // and every admission before it), not for this step's round
    if (!finishing.empty()) {
        cudaStream_t sr = wsr_.stream();
        cuda_check(cudaStreamWaitEvent(sr, step_done_, 0), "cudaStreamWaitEvent");
        std::vector<char> gone(active_.size(), 0);
        for (size_t i : finishing) {
            done.push_back(finish(active_[i]));
            gone[i] = 1;
        }
        // new states may reuse the freed memory once the frees are ordered
        // before the main stream's next allocations
        cuda_check(cudaEventRecord(freed_, sr), "cudaEventRecord");
        cuda_check(cudaStreamWaitEvent(s, freed_, 0), "cudaStreamWaitEvent");
        std::vector<Req> keep;
        keep.reserve(active_.size());
        for (size_t i = 0; i < active_.size(); ++i)
            if (!gone[i]) keep.push_back(std::move(active_[i]));
        active_.swap(keep);
    }
    const double t_adm = now();
    t_phase_[3] += t_adm - t_res;
    // 4. admit waiting requests in arrival order, once prepared, while memory
    // and slots allow; they join the next round
    while (!queue_.empty() && (int)active_.size() < max_active_ && bytes_in_use_ + queue_.front().bytes <= budget_ &&
           queue_.front().prep->ready.load(std::memory_order_acquire)) {
        Req r = std::move(queue_.front());
        queue_.pop_front();
        {
            std::lock_guard<std::mutex> lk(mu_);
            --prepared_waiting_;
        }
        cv_work_.notify_one();
        if (r.prep->error) std::rethrow_exception(r.prep->error);
        cuda_check(cudaMallocAsync(&r.state, r.bytes, s), "cudaMallocAsync(state)");
        cuda_check(cudaMemsetAsync(r.state, 0, r.bytes, s), "cudaMemsetAsync");
        cuda_check(fill_value(arith_, r.state, 1, 1.0, 0.0, s), "fill_value");
        bytes_in_use_ += r.bytes;
        r.admit_s = now();
        active_.push_back(std::move(r));
    }
    cuda_check(cudaEventRecord(step_done_, s), "cudaEventRecord");
    const double t_end = now();
    t_phase_[4] += t_end - t_adm;
    t_phase_[5] += t_end - t_start;
    return done;
}

std::vector<ServerResult> Server::drain() {
    std::vector<ServerResult> all;
    while (!queue_.empty() || !active_.empty()) {
        if (active_.empty()) {
            // nothing on the GPU: wait for the next request's preparation
            std::unique_lock<std::mutex> lk(mu_);
            cv_ready_.wait(lk, [&] { return queue_.front().prep->ready.load(std::memory_order_acquire); });
        }
        std::vector<ServerResult> d = step();
        all.insert(all.end(), d.begin(), d.end());
    }
    return all;
}

}  // namespace hqs
