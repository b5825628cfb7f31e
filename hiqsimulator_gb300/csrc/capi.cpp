// extern "C" entry points declared in include/hqs.h.
#include "../../include/hqs.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "engine.h"
#include "server.h"
#include "workspace.h"

namespace hqs {
void set_last_error(const std::string& msg);
int greedy_schedule(int ngates, const int64_t* tgt, const int* toff, const int64_t* ctl, const int* coff, int nlocals,
                    const int64_t* locals, int K, int* order, int* cluster_end);
}

struct hqs_sim {
    hqs::Engine* eng = nullptr;
    std::string err;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    std::vector<hqs::Workspace::LaunchRecord> pass_log;  // launches of the last pass_timing call
};

struct hqs_server {
    hqs::Server* srv = nullptr;
    std::string err;
    std::vector<hqs::ServerResult> pending;  // completed, not yet returned
};

struct hqs_ws {
    hqs::Workspace* ws = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
};

namespace {

thread_local std::string g_err;

}  // namespace

namespace hqs {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace hqs

namespace {

template <class F>
int guarded(std::string& err, F&& f) {
    try {
        f();
        return HQS_OK;
    } catch (const hqs::CudaError& e) {
        err = e.what();
        return HQS_ERR_CUDA;
    } catch (const std::bad_alloc& e) {
        err = "out of memory";
        return HQS_ERR_MEMORY;
    } catch (const std::invalid_argument& e) {
        err = e.what();
        return HQS_ERR_INVALID;
    } catch (const std::exception& e) {
        err = e.what();
        return HQS_ERR_RUNTIME;
    }
}

#define SIM_CALL(sim, ...)                                         \
    do {                                                           \
        if (!(sim)) {                                              \
            g_err = "null simulator handle";                       \
            return HQS_ERR_INVALID;                                \
        }                                                          \
        return guarded((sim)->err, [&]() { __VA_ARGS__; });        \
    } while (0)

void need(bool ok, const char* what) {
    if (!ok) throw std::invalid_argument(what);
}

std::vector<hqs::PauliTerm> decode_terms(size_t nterms, const size_t* off, const int64_t* idx, const char* pauli,
                                         const double* coefs) {
    need(nterms == 0 || (off && coefs), "null Pauli-term arrays");
    std::vector<hqs::PauliTerm> terms(nterms);
    for (size_t t = 0; t < nterms; ++t) {
        need(off[t] <= off[t + 1], "term offsets must not decrease");
        for (size_t f = off[t]; f < off[t + 1]; ++f) terms[t].ops.emplace_back(idx[f], pauli[f]);
        terms[t].coef = hqs::cplx(coefs[2 * t], coefs[2 * t + 1]);
    }
    return terms;
}

}  // namespace

extern "C" {

const char* hqs_last_error(void) { return g_err.c_str(); }
const char* hqs_version(void) { return "hiqsimulator_gb300 0.1 (sm_103a)"; }

int hqs_sim_create(uint64_t seed, int64_t max_local, int64_t max_cluster_size, int precision, int arith,
                   hqs_sim** out) {
    if (!out) {
        g_err = "null output pointer";
        return HQS_ERR_INVALID;
    }
    *out = nullptr;
    if (precision != HQS_C128 && precision != HQS_C64) {
        g_err = "precision must be HQS_C128 or HQS_C64";
        return HQS_ERR_INVALID;
    }
    if (arith < HQS_ARITH_AUTO || arith > HQS_ARITH_TC64) {
        g_err = "unknown arithmetic";
        return HQS_ERR_INVALID;
    }
    hqs_sim* s = new (std::nothrow) hqs_sim();
    if (!s) {
        g_err = "out of memory";
        return HQS_ERR_MEMORY;
    }
    const int rc = guarded(g_err, [&]() { s->eng = new hqs::Engine(seed, max_local, max_cluster_size, precision, arith); });
    if (rc != HQS_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return HQS_OK;
}

void hqs_sim_destroy(hqs_sim* sim) {
    if (!sim) return;
    delete sim->eng;
    if (sim->t0) cudaEventDestroy(sim->t0);
    if (sim->t1) cudaEventDestroy(sim->t1);
    delete sim;
}

const char* hqs_sim_last_error(const hqs_sim* sim) { return sim ? sim->err.c_str() : g_err.c_str(); }

int hqs_sim_allocate_qubit(hqs_sim* sim, int64_t id) { SIM_CALL(sim, sim->eng->allocate_qubit(id)); }

int hqs_sim_allocate_qureg(hqs_sim* sim, const int64_t* ids, size_t n, double init_re, double init_im) {
    SIM_CALL(sim, {
        need(n == 0 || ids, "null ids");
        sim->eng->allocate_qureg(std::vector<int64_t>(ids, ids + n), hqs::cplx(init_re, init_im));
    });
}

int hqs_sim_deallocate_qubit(hqs_sim* sim, int64_t id) { SIM_CALL(sim, sim->eng->deallocate_qubit(id)); }

int hqs_sim_apply_controlled_gate(hqs_sim* sim, const double* m, size_t dim, const int64_t* ids, size_t nids,
                                  const int64_t* ctrls, size_t nctrls) {
    SIM_CALL(sim, {
        need(m && dim > 0 && dim <= (1u << 20), "bad matrix");
        need(nids == 0 || ids, "null ids");
        need(nctrls == 0 || ctrls, "null ctrls");
        std::vector<hqs::cplx> mm(dim * dim);
        std::memcpy(static_cast<void*>(mm.data()), m, dim * dim * sizeof(hqs::cplx));
        sim->eng->apply_controlled_gate(mm, (int)dim, std::vector<int64_t>(ids, ids + nids),
                                        std::vector<int64_t>(ctrls, ctrls + nctrls));
    });
}

int hqs_sim_run(hqs_sim* sim) { SIM_CALL(sim, sim->eng->run()); }

int hqs_sim_measure_qubits(hqs_sim* sim, const int64_t* ids, size_t n, uint8_t* out) {
    SIM_CALL(sim, {
        need(n == 0 || (ids && out), "null arrays");
        const std::vector<bool> r = sim->eng->measure_qubits(std::vector<int64_t>(ids, ids + n));
        for (size_t i = 0; i < n; ++i) out[i] = r[i] ? 1 : 0;
    });
}

int hqs_sim_get_probability(hqs_sim* sim, const uint8_t* bits, size_t nbits, const int64_t* ids, size_t nids,
                            double* out) {
    SIM_CALL(sim, {
        need(out && (nids == 0 || ids) && (nbits == 0 || bits), "null arrays");
        std::vector<bool> b(nbits);
        for (size_t i = 0; i < nbits; ++i) b[i] = bits[i] != 0;
        *out = sim->eng->get_probability(b, std::vector<int64_t>(ids, ids + nids));
    });
}

int hqs_sim_get_amplitude(hqs_sim* sim, const uint8_t* bits, size_t nbits, const int64_t* ids, size_t nids,
                          double* out) {
    SIM_CALL(sim, {
        need(out && (nids == 0 || ids) && (nbits == 0 || bits), "null arrays");
        std::vector<bool> b(nbits);
        for (size_t i = 0; i < nbits; ++i) b[i] = bits[i] != 0;
        const hqs::cplx a = sim->eng->get_amplitude(b, std::vector<int64_t>(ids, ids + nids));
        out[0] = a.real();
        out[1] = a.imag();
    });
}

int hqs_sim_collapse_wavefunction(hqs_sim* sim, const int64_t* ids, size_t nids, const uint8_t* values,
                                  size_t nvalues) {
    SIM_CALL(sim, {
        need((nids == 0 || ids) && (nvalues == 0 || values), "null arrays");
        std::vector<bool> v(nvalues);
        for (size_t i = 0; i < nvalues; ++i) v[i] = values[i] != 0;
        sim->eng->collapse_wavefunction(std::vector<int64_t>(ids, ids + nids), v);
    });
}

int hqs_sim_entropy(hqs_sim* sim, double* out) {
    SIM_CALL(sim, {
        need(out, "null output");
        *out = sim->eng->entropy();
    });
}

int hqs_sim_num_qubits(const hqs_sim* sim, size_t* out) {
    if (!sim || !out) return HQS_ERR_INVALID;
    *out = sim->eng->num_qubits();
    return HQS_OK;
}

static int copy_ids(const std::vector<int64_t>& v, int64_t* out, size_t cap, size_t* n) {
    if (n) *n = v.size();
    if (v.empty()) return HQS_OK;
    if (!out || cap < v.size()) return HQS_ERR_INVALID;
    std::memcpy(out, v.data(), v.size() * sizeof(int64_t));
    return HQS_OK;
}

int hqs_sim_get_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n) {
    if (!sim) return HQS_ERR_INVALID;
    return copy_ids(sim->eng->get_qubits_ids(), out, cap, n);
}
int hqs_sim_get_local_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n) {
    if (!sim) return HQS_ERR_INVALID;
    return copy_ids(sim->eng->get_local_qubits_ids(), out, cap, n);
}
int hqs_sim_get_global_qubits_ids(const hqs_sim* sim, int64_t* out, size_t cap, size_t* n) {
    if (!sim) return HQS_ERR_INVALID;
    return copy_ids(sim->eng->get_global_qubits_ids(), out, cap, n);
}

int hqs_sim_set_qubits_perm(hqs_sim* sim, const int64_t* ids, size_t n) {
    SIM_CALL(sim, {
        need(n == 0 || ids, "null ids");
        sim->eng->set_qubits_perm(std::vector<int64_t>(ids, ids + n));
    });
}

int hqs_sim_swap_qubits(hqs_sim* sim, const int64_t* pairs, size_t n) {
    SIM_CALL(sim, {
        need(n == 0 || pairs, "null pairs");
        sim->eng->swap_qubits(std::vector<int64_t>(pairs, pairs + n));
    });
}

int hqs_sim_cheat_local(hqs_sim* sim, double* out, size_t cap) {
    SIM_CALL(sim, {
        need(out, "null output");
        sim->eng->cheat_local(reinterpret_cast<hqs::cplx*>(out), cap);
    });
}

int hqs_sim_emulate_math(hqs_sim* sim) {
    SIM_CALL(sim, throw std::runtime_error("SimulatorMPI::emulate_math() is not supported"));
}

int hqs_sim_get_expectation_value(hqs_sim* sim, size_t nterms, const size_t* term_off, const int64_t* factor_index,
                                  const char* factor_pauli, const double* coefs, const int64_t* ids, size_t nids,
                                  double* out) {
    SIM_CALL(sim, {
        need(out && (nids == 0 || ids), "null arrays");
        const auto terms = decode_terms(nterms, term_off, factor_index, factor_pauli, coefs);
        *out = sim->eng->get_expectation_value(terms, std::vector<int64_t>(ids, ids + nids));
    });
}

int hqs_sim_get_expectation_values(hqs_sim* sim, size_t nops, const size_t* op_off, const size_t* term_off,
                                   const int64_t* factor_index, const char* factor_pauli, const double* coefs,
                                   const int64_t* ids, size_t nids, double* out) {
    SIM_CALL(sim, {
        need(nops == 0 || (op_off && out), "null arrays");
        need(nids == 0 || ids, "null ids");
        if (nops == 0) return;
        need(op_off[0] == 0, "operator offsets must start at 0");
        for (size_t o = 0; o < nops; ++o) need(op_off[o] <= op_off[o + 1], "operator offsets must not decrease");
        const auto terms = decode_terms(op_off[nops], term_off, factor_index, factor_pauli, coefs);
        std::vector<std::vector<hqs::PauliTerm>> ops(nops);
        for (size_t o = 0; o < nops; ++o) ops[o].assign(terms.begin() + op_off[o], terms.begin() + op_off[o + 1]);
        const std::vector<double> v = sim->eng->get_expectation_values(ops, std::vector<int64_t>(ids, ids + nids));
        std::copy(v.begin(), v.end(), out);
    });
}

int hqs_sim_apply_qubit_operator(hqs_sim* sim, size_t nterms, const size_t* term_off, const int64_t* factor_index,
                                 const char* factor_pauli, const double* coefs, const int64_t* ids, size_t nids) {
    SIM_CALL(sim, {
        need(nids == 0 || ids, "null ids");
        const auto terms = decode_terms(nterms, term_off, factor_index, factor_pauli, coefs);
        sim->eng->apply_qubit_operator(terms, std::vector<int64_t>(ids, ids + nids));
    });
}

int hqs_sim_set_wavefunction(hqs_sim* sim, const double* wf, size_t len, const int64_t* ids, size_t nids) {
    SIM_CALL(sim, {
        need(wf && (nids == 0 || ids), "null arrays");
        sim->eng->set_wavefunction(reinterpret_cast<const hqs::cplx*>(wf), len, std::vector<int64_t>(ids, ids + nids));
    });
}

int hqs_sim_synchronize(hqs_sim* sim) { SIM_CALL(sim, sim->eng->synchronize()); }

int hqs_sim_sample(hqs_sim* sim, uint64_t shots, uint64_t* out) {
    SIM_CALL(sim, {
        need(shots == 0 || out, "null output");
        sim->eng->sample(shots, out);
    });
}

int hqs_sim_move_qubits(hqs_sim* sim, const int64_t* ids, const int* positions, size_t n) {
    SIM_CALL(sim, {
        need(n == 0 || (ids && positions), "null arrays");
        sim->eng->move_qubits(std::vector<int64_t>(ids, ids + n), std::vector<int>(positions, positions + n));
    });
}

int hqs_sim_set_pass_limits(hqs_sim* sim, int max_tile_bits, int max_ops, int defer) {
    SIM_CALL(sim, sim->eng->set_pass_limits(max_tile_bits, max_ops, defer));
}

int hqs_sim_stats(const hqs_sim* sim, uint64_t out[6]) {
    if (!sim || !out) return HQS_ERR_INVALID;
    const hqs::EngineStats& s = sim->eng->stats();
    out[0] = s.gates;
    out[1] = s.runs;
    out[2] = s.passes;
    out[3] = s.pass_ops;
    out[4] = s.bytes_moved;
    out[5] = s.flushes;
    return HQS_OK;
}

int hqs_sim_info(const hqs_sim* sim, int* precision, int* arith) {
    if (!sim) return HQS_ERR_INVALID;
    if (precision) *precision = sim->eng->precision();
    if (arith) *arith = sim->eng->arith();
    return HQS_OK;
}

int hqs_sim_state_view(hqs_sim* sim, void** state, uint64_t* amplitudes, int* device) {
    SIM_CALL(sim, {
        need(state && amplitudes, "null output");
        sim->eng->synchronize();
        void* p = sim->eng->device_state();
        cudaPointerAttributes attr{};
        hqs::cuda_check(cudaPointerGetAttributes(&attr, p), "cudaPointerGetAttributes");
        *state = p;
        *amplitudes = 1ULL << sim->eng->num_qubits();
        if (device) *device = attr.device;
    });
}

int hqs_sim_timer_start(hqs_sim* sim) {
    SIM_CALL(sim, {
        sim->eng->flush();
        if (!sim->t0) hqs::cuda_check(cudaEventCreate(&sim->t0), "cudaEventCreate");
        if (!sim->t1) hqs::cuda_check(cudaEventCreate(&sim->t1), "cudaEventCreate");
        hqs::cuda_check(cudaEventRecord(sim->t0, sim->eng->stream()), "cudaEventRecord");
    });
}

int hqs_sim_timer_stop(hqs_sim* sim, float* ms) {
    SIM_CALL(sim, {
        need(ms && sim->t0, "timer not started");
        sim->eng->flush();
        hqs::cuda_check(cudaEventRecord(sim->t1, sim->eng->stream()), "cudaEventRecord");
        hqs::cuda_check(cudaEventSynchronize(sim->t1), "cudaEventSynchronize");
        hqs::cuda_check(cudaEventElapsedTime(ms, sim->t0, sim->t1), "cudaEventElapsedTime");
    });
}

int hqs_sim_set_pass_timing(hqs_sim* sim, int on) {
    SIM_CALL(sim, {
        sim->eng->flush();
        sim->eng->workspace().set_timing(on != 0);
    });
}

int hqs_sim_pass_timing(hqs_sim* sim, uint64_t* launches, uint64_t* bytes, double* ms) {
    SIM_CALL(sim, {
        sim->eng->flush();
        hqs::Workspace::PassTiming t = sim->eng->workspace().collect_timing();
        if (launches) *launches = t.launches;
        if (bytes) *bytes = t.bytes;
        if (ms) *ms = t.ms;
        sim->pass_log = std::move(t.log);
    });
}

int hqs_sim_pass_log(hqs_sim* sim, hqs_pass_record* out, size_t cap, size_t* count) {
    SIM_CALL(sim, {
        need(count != nullptr && (cap == 0 || out != nullptr), "hqs_sim_pass_log: null output");
        *count = sim->pass_log.size();
        for (size_t i = 0; i < std::min(cap, sim->pass_log.size()); ++i) {
            const auto& r = sim->pass_log[i];
            out[i].kernel = r.kind;
            out[i].nops = r.nops;
            out[i].copies = r.copies;
            out[i].pad = 0;
            out[i].target_mask = r.target_mask;
            out[i].bytes = r.bytes;
            out[i].ms = r.ms;
        }
    });
}

int hqs_greedy_schedule(int ngates, const int64_t* tgt, const int* toff, const int64_t* ctl, const int* coff,
                        int nlocals, const int64_t* locals, int cluster_size, int* order, int* cluster_end,
                        int* nclusters) {
    return guarded(g_err, [&]() {
        need(ngates >= 0 && toff && coff && nclusters, "bad schedule arguments");
        need(ngates == 0 || (order && cluster_end), "null outputs");
        const int nc = hqs::greedy_schedule(ngates, tgt, toff, ctl, coff, nlocals, locals, cluster_size, order,
                                            cluster_end);
        if (nc < 0) throw std::runtime_error("CalcPos(): scheduling with 64 or more qubits is not yet supported");
        *nclusters = nc;
    });
}

int hqs_fuse(size_t ngates, const double* m, const size_t* dim, const int64_t* ids, const size_t* ioff,
             const int64_t* ctrls, const size_t* coff, double* out_m, size_t cap_m, int64_t* out_ids,
             size_t cap_ids, size_t* n_ids, int64_t* out_ctrls, size_t cap_ctrls, size_t* n_ctrls, int* out_diag) {
    return guarded(g_err, [&]() {
        need(ngates == 0 || (m && dim && ioff && coff), "null gate arrays");
        need(out_m && n_ids && n_ctrls && out_diag, "null outputs");
        hqs::Fusion f;
        size_t moff = 0;
        for (size_t g = 0; g < ngates; ++g) {
            need(ioff[g] <= ioff[g + 1] && coff[g] <= coff[g + 1], "offsets must not decrease");
            const size_t nt = ioff[g + 1] - ioff[g], nc = coff[g + 1] - coff[g];
            need(nt == 0 || ids, "null ids");
            need(nc == 0 || ctrls, "null ctrls");
            need(nt <= 12 && dim[g] == ((size_t)1 << nt), "a gate's matrix must be 2^targets square");
            hqs::DenseGate dg;
            dg.dim = (int)dim[g];
            dg.m.resize(dim[g] * dim[g]);
            std::memcpy(static_cast<void*>(dg.m.data()), m + 2 * moff, dg.m.size() * sizeof(hqs::cplx));
            moff += dg.m.size();
            dg.diag = hqs::is_diagonal(dg.m, dg.dim);
            if (nt) dg.ids.assign(ids + ioff[g], ids + ioff[g + 1]);
            f.insert(std::move(dg), nc ? std::vector<int64_t>(ctrls + coff[g], ctrls + coff[g + 1])
                                       : std::vector<int64_t>());
            need(f.num_qubits() <= 12, "at most 12 fused qubits");
        }
        hqs::DenseGate out;
        std::vector<int64_t> oc;
        f.perform(out, oc);
        need((size_t)out.dim * out.dim <= cap_m && out.ids.size() <= cap_ids && oc.size() <= cap_ctrls,
             "output buffers too small");
        need(out.ids.empty() || out_ids, "null output ids");
        need(oc.empty() || out_ctrls, "null output ctrls");
        std::memcpy(out_m, out.m.data(), out.m.size() * sizeof(hqs::cplx));
        std::copy(out.ids.begin(), out.ids.end(), out_ids);
        std::copy(oc.begin(), oc.end(), out_ctrls);
        *n_ids = out.ids.size();
        *n_ctrls = oc.size();
        *out_diag = out.diag ? 1 : 0;
    });
}

// ----------------------------------------------------------- server

int hqs_server_create(int precision, int arith, uint64_t budget_bytes, int max_active, int cluster_size,
                      hqs_server** out) {
    if (!out) return HQS_ERR_INVALID;
    *out = nullptr;
    hqs_server* s = new (std::nothrow) hqs_server();
    if (!s) return HQS_ERR_MEMORY;
    const int rc = guarded(g_err, [&]() {
        need(precision == HQS_C128 || precision == HQS_C64, "precision must be HQS_C128 or HQS_C64");
        s->srv = new hqs::Server(precision, arith, budget_bytes, max_active, cluster_size);
    });
    if (rc != HQS_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return HQS_OK;
}

void hqs_server_destroy(hqs_server* srv) {
    if (!srv) return;
    delete srv->srv;
    delete srv;
}

const char* hqs_server_last_error(const hqs_server* srv) { return srv ? srv->err.c_str() : g_err.c_str(); }

int hqs_server_submit(hqs_server* srv, int n, int ngates, const int* ntgt, const int* tgt, const int* nctl,
                      const int* ctl, const double* mats, int kind, double rnd, size_t nterms, const uint64_t* px,
                      const uint64_t* py, const uint64_t* pz, const double* coefs, uint64_t* id_out) {
    if (!srv) return HQS_ERR_INVALID;
    return guarded(srv->err, [&]() {
        need(ngates >= 0 && (ngates == 0 || (ntgt && nctl && mats)), "null gate arrays");
        need(kind >= HQS_RESULT_AMPLITUDE0 && kind <= HQS_RESULT_EXPECTATION, "unknown result kind");
        std::vector<hqs::ServerGate> gates(ngates);
        size_t ti = 0, ci = 0, mi = 0;
        for (int g = 0; g < ngates; ++g) {
            need(ntgt[g] >= 0 && ntgt[g] <= 10 && nctl[g] >= 0, "bad gate size");
            gates[g].targets.assign(tgt + ti, tgt + ti + ntgt[g]);
            gates[g].ctrls.assign(ctl + ci, ctl + ci + nctl[g]);
            ti += ntgt[g];
            ci += nctl[g];
            const size_t dim = (size_t)1 << ntgt[g];
            gates[g].m.resize(dim * dim);
            std::memcpy(static_cast<void*>(gates[g].m.data()), mats + 2 * mi, dim * dim * sizeof(hqs::cplx));
            mi += dim * dim;
        }
        std::vector<uint64_t> x, y, z;
        std::vector<hqs::cplx> c;
        if (kind == HQS_RESULT_EXPECTATION) {
            need(nterms == 0 || (px && py && pz && coefs), "null Pauli arrays");
            x.assign(px, px + nterms);
            y.assign(py, py + nterms);
            z.assign(pz, pz + nterms);
            for (size_t t = 0; t < nterms; ++t) c.emplace_back(coefs[2 * t], coefs[2 * t + 1]);
        }
        const uint64_t id = srv->srv->submit(n, gates, kind, rnd, x, y, z, c);
        if (id_out) *id_out = id;
    });
}

int hqs_server_step(hqs_server* srv, hqs_server_result* out, size_t cap, size_t* n) {
    if (!srv) return HQS_ERR_INVALID;
    return guarded(srv->err, [&]() {
        if (srv->pending.empty() || cap == 0) {
            std::vector<hqs::ServerResult> r = srv->srv->step();
            srv->pending.insert(srv->pending.end(), r.begin(), r.end());
        }
        size_t k = std::min(cap, srv->pending.size());
        for (size_t i = 0; i < k; ++i) {
            const hqs::ServerResult& r = srv->pending[i];
            out[i].id = r.id;
            out[i].kind = r.kind;
            out[i].value_re = r.value_re;
            out[i].value_im = r.value_im;
            out[i].sample = r.sample;
            out[i].submit_s = r.submit_s;
            out[i].admit_s = r.admit_s;
            out[i].done_s = r.done_s;
            out[i].passes = r.passes;
        }
        srv->pending.erase(srv->pending.begin(), srv->pending.begin() + k);
        if (n) *n = k;
    });
}

int hqs_server_info(const hqs_server* srv, uint64_t out[5]) {
    if (!srv || !out) return HQS_ERR_INVALID;
    out[0] = srv->srv->queued();
    out[1] = srv->srv->active();
    out[2] = srv->srv->bytes_in_use();
    out[3] = srv->srv->rounds();
    out[4] = srv->srv->launches();
    return HQS_OK;
}

int hqs_server_timing(const hqs_server* srv, double out[6]) {
    if (!srv || !out) return HQS_ERR_INVALID;
    srv->srv->timing(out);
    return HQS_OK;
}

// ----------------------------------------------------------- kernel level

int hqs_ws_create(hqs_ws** out) {
    if (!out) return HQS_ERR_INVALID;
    *out = nullptr;
    hqs_ws* w = new (std::nothrow) hqs_ws();
    if (!w) return HQS_ERR_MEMORY;
    const int rc = guarded(g_err, [&]() { w->ws = new hqs::Workspace(); });
    if (rc != HQS_OK) {
        delete w;
        return rc;
    }
    *out = w;
    return HQS_OK;
}

void hqs_ws_destroy(hqs_ws* ws) {
    if (!ws) return;
    delete ws->ws;
    if (ws->t0) cudaEventDestroy(ws->t0);
    if (ws->t1) cudaEventDestroy(ws->t1);
    delete ws;
}

#define WS_CALL(w, ...)                                  \
    do {                                                 \
        if (!(w)) {                                      \
            g_err = "null workspace";                    \
            return HQS_ERR_INVALID;                      \
        }                                                \
        return guarded(g_err, [&]() { __VA_ARGS__; });   \
    } while (0)

static void check_state_args(const void* state, int n, int arith) {
    need(state != nullptr, "null state");
    need(n >= 0 && n <= 40, "n out of range");
    need(arith >= HQS_ARITH_F64 && arith <= HQS_ARITH_TC64, "unknown arithmetic");
}

// Gates in the kernel-level array form (see hqs_apply_gates) as GateOps;
// mats may be null (zero matrices of the right sizes, for planning only).
static std::vector<hqs::GateOp> ops_from_arrays(int n, int nops, const int* k, const int* pos, const uint64_t* ctrl,
                                                const int* diag, const double* mats) {
    std::vector<hqs::GateOp> ops(nops);
    size_t off = 0;
    for (int i = 0; i < nops; ++i) {
        hqs::GateOp& op = ops[i];
        need(k[i] >= 0 && k[i] <= hqs::kMaxK && k[i] <= n, "gate size out of range");
        op.k = k[i];
        op.diag = diag[i] != 0;
        op.ctrl_mask = (k[i] == 0) ? 0 : ctrl[i];
        uint64_t seen = 0;
        for (int j = 0; j < k[i]; ++j) {
            const int p = pos[5 * i + j];
            need(p >= 0 && p < n, "target position out of range");
            need(!((seen >> p) & 1ULL), "repeated target position");
            need(!((op.ctrl_mask >> p) & 1ULL), "a target is also a control");
            seen |= 1ULL << p;
            op.pos[j] = p;
        }
        need(n >= 64 || (op.ctrl_mask >> n) == 0, "control position out of range");
        const size_t cnt = (k[i] == 0) ? 1 : (op.diag ? (1u << k[i]) : (1u << (2 * k[i])));
        op.m.assign(cnt, hqs::cplx(0.0, 0.0));
        if (mats) std::memcpy(static_cast<void*>(op.m.data()), mats + 2 * off, cnt * sizeof(hqs::cplx));
        off += cnt;
    }
    return ops;
}

int hqs_plan_passes(int n, int arith, int nops, const int* k, const int* pos, const uint64_t* ctrl, const int* diag,
                    int max_tile_bits, int max_ops, hqs_pass_info* out, size_t cap, size_t* npasses) {
    return guarded(g_err, [&]() {
        need(n >= 1 && n <= 40, "n out of range");
        need(arith >= HQS_ARITH_F64 && arith <= HQS_ARITH_TC64, "unknown arithmetic");
        need(nops >= 0 && (nops == 0 || (k && pos && ctrl && diag)), "null gate arrays");
        need(npasses && (cap == 0 || out), "null output");
        const std::vector<hqs::GateOp> ops = ops_from_arrays(n, nops, k, pos, ctrl, diag, nullptr);
        std::vector<size_t> first;
        const std::vector<hqs::PassPlan> plans = hqs::plan_passes(
            n, arith, ops, max_tile_bits > 0 ? max_tile_bits : 11, max_ops > 0 ? max_ops : 16, &first);
        *npasses = plans.size();
        for (size_t p = 0; p < plans.size() && p < cap; ++p) {
            const hqs::PassDesc& d = plans[p].desc;
            hqs_pass_info& o = out[p];
            o.first_op = (uint32_t)first[p];
            o.nops = (uint32_t)d.nops;
            o.q = (uint32_t)d.q;
            o.w = (uint32_t)d.w;
            o.prefetch = d.prefetch;
            o.tc_ops = 0;
            for (int i = 0; i < d.nops; ++i) o.tc_ops += d.ops[i].tc;
            o.tile_mask = 0;
            for (int i = 0; i < d.q; ++i) o.tile_mask |= 1ULL << d.tile_pos[i];
            o.fixed_mask = d.fixed_mask;
            o.smem_bytes = hqs::pass_smem_bytes(arith, d);
            o.pool_bytes = hqs::pass_pool_bytes(arith, d);
            o.sweep_bytes = plans[p].bytes;
        }
    });
}

int hqs_plan_launches(int n, int arith, int nops, const int* k, const int* pos, const uint64_t* ctrl, const int* diag,
                      int max_tile_bits, int max_ops, hqs_launch_info* out, size_t cap, size_t* nlaunches) {
    return guarded(g_err, [&]() {
        need(n >= 1 && n <= 40, "n out of range");
        need(arith >= HQS_ARITH_F64 && arith <= HQS_ARITH_TC64, "unknown arithmetic");
        need(nops >= 0 && (nops == 0 || (k && pos && ctrl && diag)), "null gate arrays");
        need(nlaunches && (cap == 0 || out), "null output");
        std::vector<hqs::GateOp> ops = ops_from_arrays(n, nops, k, pos, ctrl, diag, nullptr);
        for (auto& op : ops) op.m.resize(op.diag ? ((size_t)1 << op.k) : op.k == 0 ? 1 : ((size_t)1 << (2 * op.k)));
        const std::vector<hqs::LaunchPlan> L = hqs::plan_launches(
            n, arith, ops, max_tile_bits > 0 ? max_tile_bits : 11, max_ops > 0 ? max_ops : 16, hqs::umma_enabled());
        *nlaunches = L.size();
        for (size_t i = 0; i < L.size() && i < cap; ++i) {
            hqs_launch_info& o = out[i];
            std::memset(&o, 0, sizeof(o));
            const hqs::PassDesc& d = L[i].umma ? L[i].udesc.d : L[i].pass.desc;
            o.first_op = (uint32_t)L[i].first;
            o.nops = (uint32_t)d.nops;
            o.umma = L[i].umma ? 1u : 0u;
            for (int b = 0; b < d.q; ++b) o.tile_mask |= 1ULL << d.tile_pos[b];
            o.fixed_mask = d.fixed_mask;
            o.pool_bytes = L[i].pool_bytes;
            o.sweep_bytes = L[i].bytes;
            if (L[i].umma) {
                const hqs::UmmaDesc& u = L[i].udesc;
                o.tc_op = (uint32_t)u.tc_op;
                for (int j = 0; j < 5; ++j) o.target_mask |= 1ULL << d.tile_pos[u.tslot[j]];
                o.rank = u.rank;
                o.nextra = u.nextra;
                o.box_bytes = u.box_bytes;
                for (int j = 0; j < 5; ++j) {
                    o.dim_kind[j] = j < u.rank ? u.dim_kind[j] : -1;
                    o.dim_pos[j] = u.dim_pos[j];
                    o.dim_bits[j] = u.dim_bits[j];
                    o.dim_box[j] = u.dim_box[j];
                }
            }
        }
    });
}

int hqs_apply_gates(hqs_ws* ws, void* state, int n, int arith, int nops, const int* k, const int* pos,
                    const uint64_t* ctrl, const int* diag, const double* mats, int max_tile_bits, int max_ops,
                    uint64_t* bytes_out, uint64_t* passes_out) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        need(nops >= 0 && (nops == 0 || (k && pos && ctrl && diag && mats)), "null gate arrays");
        std::vector<hqs::GateOp> ops = ops_from_arrays(n, nops, k, pos, ctrl, diag, mats);
        uint64_t passes = 0;
        const uint64_t bytes = ws->ws->apply_ops(state, n, arith, ops, max_tile_bits > 0 ? max_tile_bits : 11,
                                                 max_ops > 0 ? max_ops : 16, &passes);
        if (bytes_out) *bytes_out = bytes;
        if (passes_out) *passes_out = passes;
    });
}

int hqs_probability(hqs_ws* ws, const void* state, int n, int arith, uint64_t mask, uint64_t val, double* out) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        need(out, "null output");
        need(n >= 64 || (mask >> n) == 0, "mask out of range");
        hqs::cuda_check(hqs::reduce_probability(arith, state, n, mask, val & mask, ws->ws->reduce(), ws->ws->stream(), out),
                        "reduce_probability");
    });
}

int hqs_block_sums(hqs_ws* ws, const void* state, int n, int arith, uint64_t nblocks, double* out) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        need(out && nblocks > 0 && nblocks <= (1ULL << n) && ((1ULL << n) % nblocks) == 0, "bad block count");
        double* d = static_cast<double*>(ws->ws->scratch(nblocks * sizeof(double)));
        hqs::cuda_check(hqs::block_sums(arith, state, n, nblocks, d, ws->ws->stream()), "block_sums");
        hqs::cuda_check(cudaMemcpyAsync(out, d, nblocks * sizeof(double), cudaMemcpyDeviceToHost, ws->ws->stream()),
                        "cudaMemcpyAsync");
        hqs::cuda_check(cudaStreamSynchronize(ws->ws->stream()), "cudaStreamSynchronize");
    });
}

int hqs_collapse(hqs_ws* ws, void* state, int n, int arith, uint64_t mask, uint64_t val, double scale) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        hqs::cuda_check(hqs::collapse_scale(arith, state, n, mask, val & mask, scale, ws->ws->stream()), "collapse_scale");
    });
}

int hqs_permute_bits(hqs_ws* ws, void* state, int n, int arith, int m, const uint8_t* oldpos, const uint8_t* newpos) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        need(m >= 0 && m <= hqs::kMaxTileBits && (m == 0 || (oldpos && newpos)), "bad permutation size");
        uint64_t a = 0, b = 0;
        for (int j = 0; j < m; ++j) {
            need(oldpos[j] < n && newpos[j] < n, "position out of range");
            need(!((a >> oldpos[j]) & 1ULL) && !((b >> newpos[j]) & 1ULL), "repeated position");
            a |= 1ULL << oldpos[j];
            b |= 1ULL << newpos[j];
        }
        need(a == b, "old and new positions must be the same set");
        hqs::cuda_check(hqs::permute_bits(arith, state, n, m, oldpos, newpos, ws->ws->stream()), "permute_bits");
    });
}

int hqs_drop_bit(hqs_ws* ws, void* state, int n, int arith, int pos, int keep) {
    WS_CALL(ws, {
        check_state_args(state, n, arith);
        need(n >= 1 && pos >= 0 && pos < n, "position out of range");
        hqs::cuda_check(hqs::drop_bit(arith, state, n, pos, keep ? 1 : 0, ws->ws->stream()), "drop_bit");
    });
}

int hqs_ws_synchronize(hqs_ws* ws) {
    WS_CALL(ws, ws->ws->synchronize_checked());
}

int hqs_ws_timer_start(hqs_ws* ws) {
    WS_CALL(ws, {
        if (!ws->t0) hqs::cuda_check(cudaEventCreate(&ws->t0), "cudaEventCreate");
        if (!ws->t1) hqs::cuda_check(cudaEventCreate(&ws->t1), "cudaEventCreate");
        hqs::cuda_check(cudaEventRecord(ws->t0, ws->ws->stream()), "cudaEventRecord");
    });
}

int hqs_ws_timer_stop(hqs_ws* ws, float* ms) {
    WS_CALL(ws, {
        need(ms && ws->t0, "timer not started");
        hqs::cuda_check(cudaEventRecord(ws->t1, ws->ws->stream()), "cudaEventRecord");
        hqs::cuda_check(cudaEventSynchronize(ws->t1), "cudaEventSynchronize");
        hqs::cuda_check(cudaEventElapsedTime(ms, ws->t0, ws->t1), "cudaEventElapsedTime");
    });
}

}  // extern "C"
