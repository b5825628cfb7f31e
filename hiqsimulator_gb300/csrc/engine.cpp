#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>

namespace hqs {

namespace {

std::string fmt(const char* f, ...) __attribute__((format(printf, 1, 2)));
std::string fmt(const char* f, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof(buf), f, ap);
    va_end(ap);
    return buf;
}

constexpr double kMaxFloatError = 1e-12;  // SimulatorMPI.cpp:75

}  // namespace

Engine::Engine(uint64_t seed, int64_t max_local, int64_t max_cluster_size, int precision, int arith)
    : precision_(precision == kC64 ? kC64 : kC128),
      arith_(arith),
      min_local_(max_cluster_size),
      max_local_(max_local),
      max_cluster_(max_cluster_size),
      rnd_eng_(seed) {
    if (arith_ == 0) arith_ = (precision_ == kC64) ? kArithTC64 : kArithTC;
    if (precision_ == kC64 && arith_ == kArithTC) arith_ = kArithTC64;  // tensor-core digits, two per real
    if (precision_ == kC64 && !arith_is_c64(arith_)) fail("complex64 states use F32 or TF32 arithmetic");
    if (precision_ == kC128 && arith_is_c64(arith_)) fail("complex128 states use F64, DF or TC arithmetic");
    capacity_ = 1024;
    cuda_check(cudaMalloc(&state_, capacity_ * elem_bytes()), "cudaMalloc(state)");
    cuda_check(cudaMemsetAsync(state_, 0, capacity_ * elem_bytes(), ws_.stream()), "cudaMemsetAsync");
    cuda_check(fill_value(arith_, state_, 1, 1.0, 0.0, ws_.stream()), "fill_value");  // all-zero state
    cuda_check(cudaMalloc(&block_dev_, sizeof(double) << 15), "cudaMalloc(blocks)");
    cuda_check(cudaMallocHost(&block_host_, sizeof(double) << 15), "cudaMallocHost(blocks)");
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
}

Engine::~Engine() {
    cudaStreamSynchronize(ws_.stream());
    cudaFree(state_);
    cudaFree(spare_);
    cudaFree(block_dev_);
    cudaFreeHost(block_host_);
    cudaFreeHost(scan_host_);
}

long Engine::find(int64_t id) const {
    auto it = std::find(locals_.begin(), locals_.end(), id);
    return it == locals_.end() ? -1 : (long)(it - locals_.begin());
}

// The reference looks an id up among the local qubits and then, failing that,
// with ArrayFindSure among the (here always empty) global qubits, whose error
// lists that empty array (SimulatorMPI.cpp:262-276).
size_t Engine::find_sure(int64_t id) const {
    const long p = find(id);
    if (p < 0) fail(fmt("ArrayFindSure(): Can't find %lld in ", (long long)id));
    return (size_t)p;
}

void Engine::set_pass_limits(int max_tile_bits, int max_ops, int defer) {
    if (max_tile_bits > 0) max_tile_bits_ = std::min(max_tile_bits, kMaxTileBits);
    if (max_ops > 0) max_ops_ = std::min(max_ops, kMaxOpsPerPass);
    if (defer > 0) defer_ = defer;
}

void Engine::flush() {
    if (pending_.empty()) return;
    uint64_t passes = 0;
    stats_.bytes_moved += ws_.apply_ops(state_, n(), arith_, pending_, max_tile_bits_, max_ops_, &passes);
    stats_.passes += passes;
    stats_.pass_ops += pending_.size();
    ++stats_.flushes;
    pending_.clear();
}

void Engine::synchronize() {
    flush();
    ws_.synchronize_checked();
}

void Engine::ensure_capacity(uint64_t amps) {
    if (amps <= capacity_) return;
    flush();
    uint64_t cap = amps;
    if (amps < (1ULL << 26)) cap = std::max<uint64_t>(amps, capacity_ * 2);
    void* fresh = nullptr;
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    cudaFree(spare_);
    spare_ = nullptr;
    cuda_check(cudaMalloc(&fresh, cap * elem_bytes()), "cudaMalloc(state)");
    cuda_check(cudaMemcpyAsync(fresh, state_, (1ULL << n()) * elem_bytes(), cudaMemcpyDeviceToDevice, ws_.stream()),
               "cudaMemcpyAsync(state)");
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    cudaFree(state_);
    state_ = fresh;
    capacity_ = cap;
}

void Engine::grow_one() {
    flush();
    const uint64_t N = 1ULL << n();
    ensure_capacity(2 * N);
    cuda_check(cudaMemsetAsync(static_cast<unsigned char*>(state_) + N * elem_bytes(), 0, N * elem_bytes(),
                               ws_.stream()),
               "cudaMemsetAsync");
}

// SimulatorMPI.cpp:184-216 on one rank: a new qubit always becomes local, at
// the next-highest position.
void Engine::allocate_qubit(int64_t id) {
    const int64_t local_size = (int64_t)locals_.size();
    if (local_size < min_local_ || local_size < max_local_) {
        if (locals_.size() >= 62) fail("AllocateQubit(): state vectors above 2^62 amplitudes are not supported");
        grow_one();
        locals_.push_back(id);
    } else {
        fail(fmt("AllocateQubit(): can't allocate more than %zu qubits", locals_.size()));
    }
}

// SimulatorMPI.cpp:218-251.
void Engine::allocate_qureg(const std::vector<int64_t>& ids, cplx init) {
    if (init != cplx(0.0, 0.0) && !locals_.empty())
        fail("AllocateQureg(): initialization of only first qureg is supported");
    int64_t final_n = (int64_t)locals_.size() + (int64_t)ids.size();
    const int64_t limit = std::max(min_local_, max_local_);
    if (final_n > limit) final_n = limit;
    if (final_n > (int64_t)locals_.size() && final_n < 62) ensure_capacity(1ULL << final_n);
    for (int64_t id : ids) allocate_qubit(id);
    if (init != cplx(0.0, 0.0))
        cuda_check(fill_value(arith_, state_, 1ULL << n(), init.real(), init.imag(), ws_.stream()), "fill_value");
}

// SimulatorMPI.cpp:278-322 and :369-426 on one rank.
void Engine::deallocate_qubit(int64_t id) {
    flush();
    const size_t pos = find_sure(id);
    double p[2];
    cuda_check(reduce_bit_probs(arith_, state_, n(), (int)pos, ws_.reduce(), ws_.stream(), p), "reduce_bit_probs");
    if (!((p[0] > kMaxFloatError) ^ (p[1] > kMaxFloatError)))
        fail(fmt("DeallocateLocalQubit(): qubit %lld is entangled", (long long)id));
    const int keep = (p[0] > kMaxFloatError) ? 0 : 1;
    cuda_check(drop_bit(arith_, state_, n(), (int)pos, keep, ws_.stream()), "drop_bit");
    locals_.erase(locals_.begin() + pos);
}

// SimulatorMPI.cpp:710-815 on one rank: every allocated qubit is local, so the
// global-qubit restriction of the matrix is the identity and controls on
// unallocated ids are dropped.
void Engine::apply_controlled_gate(const std::vector<cplx>& m, int dim, const std::vector<int64_t>& ids,
                                   const std::vector<int64_t>& ctrls) {
    if (dim < 1 || (size_t)dim * dim != m.size()) fail("ApplyGate(): the matrix must be square");
    if (ids.size() > 30 || dim != (1 << ids.size()))
        fail(fmt("ApplyGate(): a %dx%d matrix cannot act on %zu qubits", dim, dim, ids.size()));
    DenseGate g;
    g.dim = dim;
    g.m = m;
    g.diag = is_diagonal(m, dim);
    g.ids = ids;
    std::vector<int64_t> local_ctrls;
    for (int64_t c : ctrls)
        if (find(c) >= 0) local_ctrls.push_back(c);
    ++stats_.gates;
    if ((int64_t)(ids.size() + local_ctrls.size()) > max_cluster_) {
        run();
        fused_.insert(std::move(g), ctrls);
        return;
    }
    add_controls(g, local_ctrls);
    fused_.insert(std::move(g), {});
}

// SimulatorMPI.cpp:441-541: fuse, then queue the fused gate for the planner.
void Engine::run() {
    DenseGate g;
    std::vector<int64_t> ctrls;
    fused_.perform(g, ctrls);
    uint64_t ctrl_mask = 0;
    for (int64_t c : ctrls) {
        const long p = find(c);
        if (p >= 0) ctrl_mask |= 1ULL << p;
    }
    std::vector<int> pos(g.ids.size());
    for (size_t i = 0; i < g.ids.size(); ++i) {
        const long p = find(g.ids[i]);
        if (p < 0) {
            std::string listing;
            for (size_t j = 0; j < locals_.size(); ++j) listing += fmt("%zu:%lld ", j, (long long)locals_[j]);
            fail(fmt("ArrayFindSure(): Can't find %lld in ", (long long)g.ids[i]) + listing);
        }
        pos[i] = (int)p;
    }
    if (g.ids.size() > (size_t)kMaxK) fail(fmt("Run(): cannot apply %zu qubits gate", g.ids.size()));
    ++stats_.runs;
    GateOp op;
    op.k = (int)g.ids.size();
    if (op.k == 0) {
        fused_.clear();
        if (g.m[0] == cplx(1.0, 0.0)) return;
        op.m = {g.m[0]};
        op.ctrl_mask = 0;  // the reference's 0-qubit kernel ignores controls
    } else {
        for (int j = 0; j < op.k; ++j) op.pos[j] = pos[j];
        op.ctrl_mask = ctrl_mask;
        op.diag = g.diag;
        if (g.diag) {
            op.m.resize(g.dim);
            for (int r = 0; r < g.dim; ++r) op.m[r] = g.m[(size_t)r * g.dim + r];
        } else {
            op.m = std::move(g.m);
        }
        fused_.clear();
    }
    pending_.push_back(std::move(op));
    if ((int)pending_.size() >= defer_) flush();
}

void Engine::masks_for(const std::vector<int64_t>& ids, const std::vector<bool>& bits, uint64_t& msk,
                       uint64_t& val) const {
    msk = val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
        const size_t pos = find_sure(ids[i]);
        msk |= 1ULL << pos;
        if (bits[i]) val |= 1ULL << pos;
    }
}

double Engine::probability_internal(uint64_t msk, uint64_t val) {
    double p = 0.0;
    cuda_check(reduce_probability(arith_, state_, n(), msk, val, ws_.reduce(), ws_.stream(), &p),
               "reduce_probability");
    return p;
}

void Engine::normalize(double norm, uint64_t msk, uint64_t val) {
    const double scale = 1.0 / std::sqrt(norm);
    cuda_check(collapse_scale(arith_, state_, n(), msk, val, scale, ws_.stream()), "collapse_scale");
}

// Block CDF (SimulatorMPI.cpp:817-839) + linear search + in-block scan
// (:921-961). Returns the sampled basis index; ok=false when rnd exceeds the
// total probability.
uint64_t Engine::sample_index(double rnd, bool& ok, double* total) {
    const uint64_t N = 1ULL << n();
    const uint64_t nb = std::min<uint64_t>(N, 1ULL << 15);
    cuda_check(block_sums(arith_, state_, n(), nb, block_dev_, ws_.stream()), "block_sums");
    cuda_check(cudaMemcpyAsync(block_host_, block_dev_, nb * sizeof(double), cudaMemcpyDeviceToHost, ws_.stream()),
               "cudaMemcpyAsync(blocks)");
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    std::partial_sum(block_host_, block_host_ + nb, block_host_);
    if (total) *total = block_host_[nb - 1];
    uint64_t i = 0;
    for (; i < nb; ++i)
        if (rnd <= block_host_[i]) break;
    if (i == nb) {
        ok = false;
        return 0;
    }
    ok = true;
    const uint64_t K = N / nb;
    if (scan_cap_ < K) {
        cudaFreeHost(scan_host_);
        scan_host_ = nullptr;
        scan_cap_ = 0;
        cuda_check(cudaMallocHost(&scan_host_, K * sizeof(cplx)), "cudaMallocHost(scan)");
        scan_cap_ = K;
    }
    if (precision_ == kC64) {
        std::vector<float> tmp(2 * K);
        cuda_check(cudaMemcpyAsync(tmp.data(), static_cast<const unsigned char*>(state_) + i * K * 8, K * 8,
                                   cudaMemcpyDeviceToHost, ws_.stream()),
                   "cudaMemcpyAsync(block)");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
        for (uint64_t j = 0; j < K; ++j) scan_host_[j] = cplx(tmp[2 * j], tmp[2 * j + 1]);
    } else {
        cuda_check(cudaMemcpyAsync(scan_host_, static_cast<const unsigned char*>(state_) + i * K * 16, K * 16,
                                   cudaMemcpyDeviceToHost, ws_.stream()),
                   "cudaMemcpyAsync(block)");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    }
    return scan_block(i, K, rnd);
}

// In-block scan (SimulatorMPI.cpp:950-958) over the host copy of block i:
// the first index whose running sum reaches rnd. The block CDF comes from
// device block sums and the scan from a host sum, so rounding can leave the
// scan just short of rnd; the draw then belongs to the block's last
// amplitude with nonzero probability (never past the block).
uint64_t Engine::scan_block(uint64_t i, uint64_t K, double rnd) const {
    double shift = (i > 0) ? block_host_[i - 1] : 0.0;
    uint64_t last = i * K;
    for (uint64_t j = 0; j < K; ++j) {
        const double p = std::norm(scan_host_[j]);
        if (p > 0.0) last = i * K + j;
        shift += p;
        if (shift >= rnd) return i * K + j;
    }
    return last;
}

// SimulatorMPI.cpp:897-1008.
std::vector<bool> Engine::measure_qubits(const std::vector<int64_t>& ids) {
    flush();
    const double rnd = dist_(rnd_eng_);
    bool ok = false;
    double total = 0.0;
    const uint64_t res_index = sample_index(rnd, ok, &total);
    if (!ok) fail(fmt("MeasureQubits(): Random number %.3f > norm partial sum %.3f", rnd, total));
    std::vector<bool> res(ids.size());
    uint64_t msk = 0, val = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
        const size_t pos = find_sure(ids[i]);
        msk |= 1ULL << pos;
        if ((res_index >> pos) & 1ULL) {
            val |= 1ULL << pos;
            res[i] = true;
        }
    }
    const double norm = probability_internal(msk, val);
    normalize(norm, msk, val);
    return res;
}

void Engine::sample(uint64_t shots, uint64_t* out) {
    flush();
    if (shots == 0) return;
    const uint64_t N = 1ULL << n();
    const uint64_t nb = std::min<uint64_t>(N, 1ULL << 15);
    const uint64_t K = N / nb;
    std::vector<double> rnd(shots);
    for (auto& r : rnd) r = dist_(rnd_eng_);
    cuda_check(block_sums(arith_, state_, n(), nb, block_dev_, ws_.stream()), "block_sums");
    cuda_check(cudaMemcpyAsync(block_host_, block_dev_, nb * sizeof(double), cudaMemcpyDeviceToHost, ws_.stream()),
               "cudaMemcpyAsync(blocks)");
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    std::partial_sum(block_host_, block_host_ + nb, block_host_);
    std::vector<uint64_t> order(shots);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return rnd[a] < rnd[b]; });
    if (scan_cap_ < K) {
        cudaFreeHost(scan_host_);
        scan_host_ = nullptr;
        scan_cap_ = 0;
        cuda_check(cudaMallocHost(&scan_host_, K * sizeof(cplx)), "cudaMallocHost(scan)");
        scan_cap_ = K;
    }
    uint64_t loaded = ~0ULL;
    std::vector<float> tmp;
    for (uint64_t s : order) {
        uint64_t i = std::lower_bound(block_host_, block_host_ + nb, rnd[s]) - block_host_;
        if (i == nb) fail(fmt("MeasureQubits(): Random number %.3f > norm partial sum %.3f", rnd[s], block_host_[nb - 1]));
        if (i != loaded) {
            if (precision_ == kC64) {
                tmp.resize(2 * K);
                cuda_check(cudaMemcpy(tmp.data(), static_cast<const unsigned char*>(state_) + i * K * 8, K * 8,
                                      cudaMemcpyDeviceToHost),
                           "cudaMemcpy(block)");
                for (uint64_t j = 0; j < K; ++j) scan_host_[j] = cplx(tmp[2 * j], tmp[2 * j + 1]);
            } else {
                cuda_check(cudaMemcpyAsync(scan_host_, static_cast<const unsigned char*>(state_) + i * K * 16, K * 16,
                                           cudaMemcpyDeviceToHost, ws_.stream()),
                           "cudaMemcpyAsync(block)");
                cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
            }
            loaded = i;
        }
        out[s] = scan_block(i, K, rnd[s]);
    }
}

// SimulatorMPI.cpp:561-600.
double Engine::get_probability(const std::vector<bool>& bits, const std::vector<int64_t>& ids) {
    flush();
    if (ids.size() != bits.size()) fail("GetProbability(): ids.size() != bit_string.size()");
    uint64_t msk, val;
    masks_for(ids, bits, msk, val);
    return probability_internal(msk, val);
}

// SimulatorMPI.cpp:602-650.
cplx Engine::get_amplitude(const std::vector<bool>& bits, const std::vector<int64_t>& ids) {
    flush();
    if (bits.size() != locals_.size() || bits.size() != ids.size())
        fail("GetAmplitude(): ids.size() != number of qubits");
    uint64_t num = 0, check = 0;
    for (size_t i = 0; i < ids.size(); ++i) {
        const size_t pos = find_sure(ids[i]);
        if (bits[i]) num |= 1ULL << pos;
        check |= 1ULL << pos;
    }
    if (check != (1ULL << locals_.size()) - 1ULL)
        fail("GetAmplitude(): the second argument must be a permutation of all allocated qubits.");
    if (precision_ == kC64) {
        float v[2];
        cuda_check(cudaMemcpyAsync(v, static_cast<const unsigned char*>(state_) + num * 8, 8, cudaMemcpyDeviceToHost,
                                   ws_.stream()),
                   "cudaMemcpyAsync(amplitude)");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
        return cplx(v[0], v[1]);
    }
    double v[2];
    cuda_check(cudaMemcpyAsync(v, static_cast<const unsigned char*>(state_) + num * 16, 16, cudaMemcpyDeviceToHost,
                               ws_.stream()),
               "cudaMemcpyAsync(amplitude)");
    cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    return cplx(v[0], v[1]);
}

// SimulatorMPI.cpp:1010-1058.
void Engine::collapse_wavefunction(const std::vector<int64_t>& ids, const std::vector<bool>& values) {
    flush();
    if (ids.size() != values.size()) fail("collapseWaveFunction(): ids.size() != values.size()");
    uint64_t msk, val;
    masks_for(ids, values, msk, val);
    const double norm = probability_internal(msk, val);
    if (norm < 1.e-12) fail("collapseWaveFunction(): Invalid collapse! Probability is ~0.");
    normalize(norm, msk, val);
}

double Engine::entropy() {
    flush();
    double e = 0.0;
    cuda_check(reduce_entropy(arith_, state_, n(), ws_.reduce(), ws_.stream(), &e), "reduce_entropy");
    return e;
}

// SimulatorMPI.cpp:661-667: relabels positions without moving data.
void Engine::set_qubits_perm(const std::vector<int64_t>& p) {
    if (p.size() < locals_.size()) fail("SetQubitsPermutation(): too few qubit ids");
    flush();
    locals_.assign(p.begin(), p.begin() + locals_.size());
}

// SimulatorMPI.cpp:1085-1138: pairs are (global id, local id); one device has
// no global qubits, so any pair fails the way the reference's lookup does.
void Engine::swap_qubits(const std::vector<int64_t>& pairs) {
    if (pairs.empty()) return;
    fail(fmt("ArrayFindSure(): Can't find %lld in ", (long long)pairs[0]));
}

void Engine::cheat_local(cplx* out, size_t cap) {
    flush();
    const uint64_t N = 1ULL << n();
    if (cap < N) fail("cheat_local(): output buffer too small");
    if (precision_ == kC64) {
        std::vector<float> tmp(2 * N);
        cuda_check(cudaMemcpyAsync(tmp.data(), state_, N * 8, cudaMemcpyDeviceToHost, ws_.stream()), "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
        for (uint64_t i = 0; i < N; ++i) out[i] = cplx(tmp[2 * i], tmp[2 * i + 1]);
    } else {
        cuda_check(cudaMemcpyAsync(out, state_, N * 16, cudaMemcpyDeviceToHost, ws_.stream()), "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    }
}

void Engine::pauli_masks(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids, std::vector<uint64_t>& xm,
                         std::vector<uint64_t>& ym, std::vector<uint64_t>& zm) const {
    for (const auto& t : terms) {
        uint64_t x = 0, y = 0, z = 0, seen = 0;
        for (const auto& o : t.ops) {
            if (o.first < 0 || (size_t)o.first >= ids.size())
                fail("qubit_operator acts on more qubits than contained in the qureg.");
            const uint64_t b = 1ULL << find_sure(ids[o.first]);
            if (seen & b) fail("a Pauli term names the same qubit twice");
            seen |= b;
            switch (o.second) {
                case 'X': x |= b; break;
                case 'Y': x |= b; y |= b; break;
                case 'Z': z |= b; break;
                default: fail(fmt("unknown Pauli operator '%c'", o.second));
            }
        }
        xm.push_back(x);
        ym.push_back(y);
        zm.push_back(z);
    }
}

// Sum_t Re(c_t <psi|P_t|psi>) over Pauli strings P_t on qubits ids[index]
// (semantics of get_expectation_value, hiq/projectq/backends/_sim/_simulator_mpi.py:148-183).
double Engine::get_expectation_value(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids) {
    run();
    flush();
    std::vector<uint64_t> xm, ym, zm;
    pauli_masks(terms, ids, xm, ym, zm);
    if (terms.empty()) return 0.0;
    const size_t T = terms.size();
    if (T == 1 && xm[0] == 0) {
        // one Z string: <psi|Z..Z|psi> is real, Re(c <.>) = Re(c) <.>
        double out = 0.0;
        cuda_check(reduce_pauli_expectation(arith_, state_, n(), 1, nullptr, nullptr, nullptr, nullptr, ws_.reduce(),
                                            ws_.stream(), &out, true, zm[0]),
                   "reduce_pauli_expectation");
        return terms[0].coef.real() * out;
    }
    std::vector<unsigned char> blob(T * (3 * 8 + 16));
    std::memcpy(blob.data(), xm.data(), T * 8);
    std::memcpy(blob.data() + T * 8, ym.data(), T * 8);
    std::memcpy(blob.data() + 2 * T * 8, zm.data(), T * 8);
    double* co = reinterpret_cast<double*>(blob.data() + 3 * T * 8);
    for (size_t t = 0; t < T; ++t) {
        co[2 * t] = terms[t].coef.real();
        co[2 * t + 1] = terms[t].coef.imag();
    }
    const unsigned char* d = static_cast<const unsigned char*>(ws_.upload(blob.data(), blob.size()));
    double out = 0.0;
    cuda_check(reduce_pauli_expectation(arith_, state_, n(), (int)T, (const uint64_t*)d, (const uint64_t*)(d + T * 8),
                                        (const uint64_t*)(d + 2 * T * 8), (const double*)(d + 3 * T * 8), ws_.reduce(),
                                        ws_.stream(), &out),
               "reduce_pauli_expectation");
    return out;
}

std::vector<double> Engine::get_expectation_values(const std::vector<std::vector<PauliTerm>>& ops,
                                                   const std::vector<int64_t>& ids) {
    run();
    flush();
    std::vector<double> out(ops.size(), 0.0);
    std::vector<uint64_t> masks;  // distinct Z strings of the Z-only operators
    std::map<uint64_t, size_t> slot;
    std::vector<std::vector<uint64_t>> zterms(ops.size());
    std::vector<char> zonly(ops.size(), 0);
    for (size_t o = 0; o < ops.size(); ++o) {
        std::vector<uint64_t> xm, ym, zm;
        pauli_masks(ops[o], ids, xm, ym, zm);
        bool z = true;
        for (uint64_t x : xm) z = z && x == 0;
        if (!z) {
            out[o] = get_expectation_value(ops[o], ids);
            continue;
        }
        zonly[o] = 1;
        zterms[o] = zm;
        for (uint64_t m : zm)
            if (slot.emplace(m, masks.size()).second) masks.push_back(m);
    }
    // <Z string> = sum_i (-1)^popcount(i & z) |a_i|^2 (real); Re(c <P>) = Re(c) <P>
    std::vector<double> val(masks.size(), 0.0);
    for (size_t b = 0; b < masks.size(); b += 64) {
        const int T = (int)std::min<size_t>(64, masks.size() - b);
        const uint64_t* d_z = static_cast<const uint64_t*>(ws_.upload(masks.data() + b, (size_t)T * 8));
        double* scratch = static_cast<double*>(ws_.scratch(zparity_multi_scratch_bytes(T)));
        cuda_check(reduce_zparity_multi(arith_, state_, n(), T, d_z, scratch, ws_.stream(), val.data() + b),
                   "reduce_zparity_multi");
    }
    for (size_t o = 0; o < ops.size(); ++o) {
        if (!zonly[o]) continue;
        double v = 0.0;
        for (size_t t = 0; t < ops[o].size(); ++t) v += ops[o][t].coef.real() * val[slot[zterms[o][t]]];
        out[o] = v;
    }
    return out;
}

// psi <- sum_t c_t P_t psi without renormalisation (semantics of
// apply_qubit_operator, hiq/projectq/backends/_sim/_simulator_mpi.py:185-223).
void Engine::apply_qubit_operator(const std::vector<PauliTerm>& terms, const std::vector<int64_t>& ids) {
    run();
    flush();
    std::vector<uint64_t> xm, ym, zm;
    pauli_masks(terms, ids, xm, ym, zm);
    const size_t T = terms.size();
    const uint64_t N = 1ULL << n();
    if (T == 0) {
        cuda_check(cudaMemsetAsync(state_, 0, N * elem_bytes(), ws_.stream()), "cudaMemsetAsync");
        return;
    }
    const size_t melem = Workspace::mat_elem_bytes(arith_);
    // coefficient table starts on a 256-byte boundary (16-byte vector loads)
    const size_t coff = (T * 3 * 8 + 255) & ~(size_t)255;
    std::vector<unsigned char> blob(coff + 2 * T * melem);
    std::memcpy(blob.data(), xm.data(), T * 8);
    std::memcpy(blob.data() + T * 8, ym.data(), T * 8);
    std::memcpy(blob.data() + 2 * T * 8, zm.data(), T * 8);
    unsigned char* cb = blob.data() + coff;
    for (size_t t = 0; t < T; ++t) {
        cplx c = terms[t].coef;
        const int ny = __builtin_popcountll(ym[t]) & 3;
        for (int r = 0; r < ny; ++r) c *= cplx(0.0, 1.0);
        for (int sgn = 0; sgn < 2; ++sgn) {
            const cplx v = sgn ? -c : c;
            unsigned char* dst = cb + (2 * t + sgn) * melem;
            if (arith_ == kArithF64) {
                double* p = reinterpret_cast<double*>(dst);
                p[0] = v.real();
                p[1] = v.imag();
            } else if (arith_ == kArithDF || arith_ == kArithTC) {
                float* p = reinterpret_cast<float*>(dst);
                p[0] = (float)v.real();
                p[1] = (float)v.imag();
                p[2] = (float)(v.real() - (double)p[0]);
                p[3] = (float)(v.imag() - (double)p[1]);
            } else {
                float* p = reinterpret_cast<float*>(dst);
                p[0] = (float)v.real();
                p[1] = (float)v.imag();
            }
        }
    }
    if (spare_cap_ < capacity_) {
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
        cudaFree(spare_);
        spare_ = nullptr;
        spare_cap_ = 0;
        cuda_check(cudaMalloc(&spare_, capacity_ * elem_bytes()), "cudaMalloc(operator buffer)");
        spare_cap_ = capacity_;
    }
    const unsigned char* d = static_cast<const unsigned char*>(ws_.upload(blob.data(), blob.size()));
    cuda_check(pauli_apply(arith_, state_, spare_, n(), (int)T, (const uint64_t*)d, (const uint64_t*)(d + T * 8),
                           (const uint64_t*)(d + 2 * T * 8), (const double*)(d + coff), ws_.stream()),
               "pauli_apply");
    std::swap(state_, spare_);
}

// Adopt the given qubit order and amplitudes (semantics of set_wavefunction,
// hiq/projectq/backends/_sim/_simulator_mpi.py:285-306).
void Engine::set_wavefunction(const cplx* wf, size_t len, const std::vector<int64_t>& ids) {
    run();
    flush();
    if (ids.size() != locals_.size())
        fail("set_wavefunction(): the qureg must contain all allocated qubits");
    std::vector<int64_t> a(ids), b(locals_);
    std::sort(a.begin(), a.end());
    std::sort(b.begin(), b.end());
    if (a != b || std::adjacent_find(a.begin(), a.end()) != a.end())
        fail("set_wavefunction(): the qureg must contain all allocated qubits");
    if (len != (1ULL << locals_.size()))
        fail("set_wavefunction(): the wavefunction must have 2^n amplitudes for n qubits");
    locals_ = ids;
    if (precision_ == kC64) {
        std::vector<float> tmp(2 * len);
        for (size_t i = 0; i < len; ++i) {
            tmp[2 * i] = (float)wf[i].real();
            tmp[2 * i + 1] = (float)wf[i].imag();
        }
        cuda_check(cudaMemcpyAsync(state_, tmp.data(), len * 8, cudaMemcpyHostToDevice, ws_.stream()), "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    } else {
        cuda_check(cudaMemcpyAsync(state_, wf, len * 16, cudaMemcpyHostToDevice, ws_.stream()), "cudaMemcpyAsync");
        cuda_check(cudaStreamSynchronize(ws_.stream()), "cudaStreamSynchronize");
    }
}

void Engine::move_qubits(const std::vector<int64_t>& ids, const std::vector<int>& positions) {
    flush();
    if (ids.size() != positions.size()) fail("move_qubits(): ids and positions differ in length");
    const int nq = n();
    std::vector<int> newpos_of(nq, -1);  // old position -> new position
    std::vector<bool> target_taken(nq, false);
    for (size_t i = 0; i < ids.size(); ++i) {
        const int o = (int)find_sure(ids[i]);
        const int p = positions[i];
        if (p < 0 || p >= nq) fail("move_qubits(): position out of range");
        if (newpos_of[o] >= 0 || target_taken[p]) fail("move_qubits(): repeated qubit or position");
        newpos_of[o] = p;
        target_taken[p] = true;
    }
    // displaced qubits fill the vacated positions in ascending order
    std::vector<int> vacated;
    for (int o = 0; o < nq; ++o)
        if (newpos_of[o] >= 0 && !target_taken[o]) vacated.push_back(o);
    size_t vi = 0;
    for (int p = 0; p < nq; ++p)
        if (target_taken[p] && newpos_of[p] < 0) newpos_of[p] = vacated[vi++];
    std::vector<uint8_t> op, np;
    for (int o = 0; o < nq; ++o)
        if (newpos_of[o] >= 0 && newpos_of[o] != o) {
            op.push_back((uint8_t)o);
            np.push_back((uint8_t)newpos_of[o]);
        }
    if (op.size() > (size_t)kMaxTileBits) fail("move_qubits(): at most 12 positions can change in one sweep");
    if (op.empty()) return;
    cuda_check(permute_bits(arith_, state_, nq, (int)op.size(), op.data(), np.data(), ws_.stream()), "permute_bits");
    std::vector<int64_t> nl(locals_);
    for (size_t j = 0; j < op.size(); ++j) nl[np[j]] = locals_[op[j]];
    locals_ = nl;
}

}  // namespace hqs
