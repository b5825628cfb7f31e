// pybind11 module `_cppsim_mpi`: the drop-in for the reference module of the
// same name (_cppsim_mpi.cpp:61-83). Class SimulatorMPI keeps the reference's
// constructor and the 17 bound method names and argument shapes, and adds the
// three methods the Python backend calls that the reference never bound
// (get_expectation_value, apply_qubit_operator, set_wavefunction). Every
// method forwards to the C ABI of libhqs.so (include/hqs.h).
#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <complex>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/hqs.h"

namespace py = pybind11;
using cplx = std::complex<double>;
using Ids = std::vector<int64_t>;

namespace {

[[noreturn]] void raise(int rc, const char* msg) {
    const std::string m = msg ? msg : "unknown error";
    switch (rc) {
        case HQS_ERR_INVALID: throw py::value_error(m);
        case HQS_ERR_MEMORY: throw std::bad_alloc();
        default: throw std::runtime_error(m);
    }
}

int parse_precision(const std::string& p) {
    if (p == "c128" || p == "complex128") return HQS_C128;
    if (p == "c64" || p == "complex64") return HQS_C64;
    throw py::value_error("precision must be 'c128' or 'c64'");
}

int parse_arith(const std::string& a) {
    if (a.empty() || a == "auto") return HQS_ARITH_AUTO;
    if (a == "f64") return HQS_ARITH_F64;
    if (a == "df") return HQS_ARITH_DF;
    if (a == "f32") return HQS_ARITH_F32;
    if (a == "tc") return HQS_ARITH_TC;
    if (a == "tf32") return HQS_ARITH_TF32;
    if (a == "tc64") return HQS_ARITH_TC64;
    throw py::value_error("arith must be 'auto', 'f64', 'df', 'tc', 'f32', 'tf32' or 'tc64'");
}

std::string env_or(const char* name, const char* dflt) {
    const char* v = std::getenv(name);
    return (v && *v) ? std::string(v) : std::string(dflt);
}

// DLPack exchange structures (unversioned ABI, DLPack 0.8), laid out as the
// DLPack specification defines them, so that torch.from_dlpack / cupy adopt
// the state without a copy from a capsule named "dltensor".
struct DLDevice {
    int32_t device_type;  // 2 = CUDA
    int32_t device_id;
};
struct DLDataType {
    uint8_t code;  // 5 = complex
    uint8_t bits;
    uint16_t lanes;
};
struct DLTensor {
    void* data;
    DLDevice device;
    int32_t ndim;
    DLDataType dtype;
    int64_t* shape;
    int64_t* strides;
    uint64_t byte_offset;
};
struct DLManagedTensor {
    DLTensor dl_tensor;
    void* manager_ctx;
    void (*deleter)(DLManagedTensor*);
};

// Owns one exported view: its shape/strides and a reference to the Python
// simulator object, which keeps the device state allocated while a consumer
// holds the view.
struct StateView {
    DLManagedTensor t{};
    int64_t shape[1] = {0};
    int64_t strides[1] = {1};
    PyObject* owner = nullptr;
};

void state_view_deleter(DLManagedTensor* t) {
    StateView* v = static_cast<StateView*>(t->manager_ctx);
    if (v->owner && Py_IsInitialized()) {
        // consumers may free the view from a thread without the GIL
        const PyGILState_STATE g = PyGILState_Ensure();
        Py_DECREF(v->owner);
        PyGILState_Release(g);
    }
    delete v;
}

// A capsule that no consumer renamed to "used_dltensor" still owns its view.
void state_capsule_destructor(PyObject* cap) {
    if (!PyCapsule_IsValid(cap, "dltensor")) return;
    auto* t = static_cast<DLManagedTensor*>(PyCapsule_GetPointer(cap, "dltensor"));
    if (t && t->deleter) t->deleter(t);
}

struct PauliArgs {
    std::vector<size_t> off{0};
    std::vector<int64_t> idx;
    std::vector<char> pauli;
    std::vector<double> coefs;
};

// op = [(term, coef), ...] with term = [(index, 'X'|'Y'|'Z'), ...]
// (the encoding built at hiq/projectq/backends/_sim/_simulator_mpi.py:180-183).
PauliArgs encode(const py::object& op) {
    PauliArgs a;
    for (py::handle item : op) {
        py::sequence pair = py::reinterpret_borrow<py::sequence>(item);
        if (py::len(pair) != 2) throw py::value_error("each operator entry must be (term, coefficient)");
        for (py::handle f : py::reinterpret_borrow<py::sequence>(pair[0])) {
            py::sequence fs = py::reinterpret_borrow<py::sequence>(f);
            a.idx.push_back(fs[0].cast<int64_t>());
            const std::string p = fs[1].cast<std::string>();
            if (p.size() != 1) throw py::value_error("Pauli factors are 'X', 'Y' or 'Z'");
            a.pauli.push_back(p[0]);
        }
        a.off.push_back(a.idx.size());
        const cplx c = pair[1].cast<cplx>();
        a.coefs.push_back(c.real());
        a.coefs.push_back(c.imag());
    }
    return a;
}

class SimulatorMPI {
public:
    SimulatorMPI(uint64_t seed, int64_t max_local, int64_t max_cluster_size, const std::string& precision,
                 const std::string& arith) {
        const int p = parse_precision(precision.empty() ? env_or("HQS_PRECISION", "c128") : precision);
        const int a = parse_arith(arith.empty() ? env_or("HQS_ARITH", "auto") : arith);
        const int rc = hqs_sim_create(seed, max_local, max_cluster_size, p, a, &h_);
        if (rc != HQS_OK) raise(rc, hqs_last_error());
    }
    ~SimulatorMPI() { hqs_sim_destroy(h_); }
    SimulatorMPI(const SimulatorMPI&) = delete;

    void check(int rc) const {
        if (rc != HQS_OK) raise(rc, hqs_sim_last_error(h_));
    }

    Ids ids_of(int (*f)(const hqs_sim*, int64_t*, size_t, size_t*)) const {
        size_t n = 0;
        check(hqs_sim_num_qubits(h_, &n));
        Ids v(n);
        size_t got = 0;
        check(f(h_, v.data(), v.size(), &got));
        v.resize(got);
        return v;
    }
    Ids get_qubits_ids() const { return ids_of(hqs_sim_get_qubits_ids); }
    Ids get_local_qubits_ids() const { return ids_of(hqs_sim_get_local_qubits_ids); }
    Ids get_global_qubits_ids() const { return ids_of(hqs_sim_get_global_qubits_ids); }
    void set_qubits_perm(const Ids& p) { check(hqs_sim_set_qubits_perm(h_, p.data(), p.size())); }
    void swap_qubits(const Ids& p) { check(hqs_sim_swap_qubits(h_, p.data(), p.size())); }
    void allocate_qureg(const Ids& ids, cplx init) {
        check(hqs_sim_allocate_qureg(h_, ids.data(), ids.size(), init.real(), init.imag()));
    }
    void allocate_qubit(int64_t id) { check(hqs_sim_allocate_qubit(h_, id)); }
    void deallocate_qubit(int64_t id) { check(hqs_sim_deallocate_qubit(h_, id)); }
    std::vector<bool> measure_qubits(const Ids& ids) {
        std::vector<uint8_t> out(ids.size());
        check(hqs_sim_measure_qubits(h_, ids.data(), ids.size(), out.data()));
        return std::vector<bool>(out.begin(), out.end());
    }
    void apply_controlled_gate(const std::vector<std::vector<cplx>>& m, const Ids& ids, const Ids& ctrls) {
        const size_t dim = m.size();
        if (dim == 0) throw std::runtime_error("ApplyGate(): empty matrix");
        std::vector<cplx> flat(dim * dim);
        for (size_t r = 0; r < dim; ++r) {
            if (m[r].size() != dim) throw std::runtime_error("ApplyGate(): the matrix must be square");
            std::memcpy(static_cast<void*>(&flat[r * dim]), m[r].data(), dim * sizeof(cplx));
        }
        check(hqs_sim_apply_controlled_gate(h_, reinterpret_cast<const double*>(flat.data()), dim, ids.data(),
                                            ids.size(), ctrls.data(), ctrls.size()));
    }
    void emulate_math(const py::object&, const py::object&, const py::object&) { check(hqs_sim_emulate_math(h_)); }
    void emulate_time_evolution(const py::object&, const py::object&, const py::object&, const py::object&) {
        throw std::runtime_error("SimulatorMPI::emulate_time_evolution() is not supported");
    }
    cplx get_amplitude(const std::vector<bool>& bits, const Ids& ids) {
        std::vector<uint8_t> b(bits.begin(), bits.end());
        double out[2];
        check(hqs_sim_get_amplitude(h_, b.data(), b.size(), ids.data(), ids.size(), out));
        return cplx(out[0], out[1]);
    }
    double get_probability(const std::vector<bool>& bits, const Ids& ids) {
        std::vector<uint8_t> b(bits.begin(), bits.end());
        double out = 0;
        check(hqs_sim_get_probability(h_, b.data(), b.size(), ids.data(), ids.size(), &out));
        return out;
    }
    void run() { check(hqs_sim_run(h_)); }
    double entropy() {
        double e = 0;
        check(hqs_sim_entropy(h_, &e));
        return e;
    }
    std::map<int, int> id2pos() const {
        std::map<int, int> m;
        const Ids ids = get_qubits_ids();
        for (size_t p = 0; p < ids.size(); ++p) m[(int)ids[p]] = (int)p;
        return m;
    }
    std::vector<cplx> state() {
        size_t n = 0;
        check(hqs_sim_num_qubits(h_, &n));
        std::vector<cplx> v((size_t)1 << n);
        check(hqs_sim_cheat_local(h_, reinterpret_cast<double*>(v.data()), v.size()));
        return v;
    }
    std::tuple<std::map<int, int>, std::vector<cplx>> cheat_local() { return {id2pos(), state()}; }
    std::tuple<std::map<int, int>, py::array_t<cplx>> cheat_local_numpy() {
        size_t n = 0;
        check(hqs_sim_num_qubits(h_, &n));
        py::array_t<cplx> a((py::ssize_t)((size_t)1 << n));
        check(hqs_sim_cheat_local(h_, reinterpret_cast<double*>(a.mutable_data()), (size_t)a.size()));
        return {id2pos(), a};
    }
    void collapse_wavefunction(const Ids& ids, const std::vector<bool>& values) {
        std::vector<uint8_t> v(values.begin(), values.end());
        check(hqs_sim_collapse_wavefunction(h_, ids.data(), ids.size(), v.data(), v.size()));
    }
    double get_expectation_value(const py::object& op, const Ids& ids) {
        const PauliArgs a = encode(op);
        double out = 0;
        check(hqs_sim_get_expectation_value(h_, a.off.size() - 1, a.off.data(), a.idx.data(), a.pauli.data(),
                                            a.coefs.data(), ids.data(), ids.size(), &out));
        return out;
    }
    // one value per operator; Z-only operators share one read of the state per 64 Z strings
    std::vector<double> get_expectation_values(const py::object& ops, const Ids& ids) {
        PauliArgs all;
        std::vector<size_t> op_off{0};
        for (py::handle op : ops) {
            const PauliArgs a = encode(py::reinterpret_borrow<py::object>(op));
            const size_t base = all.idx.size();
            for (size_t t = 1; t < a.off.size(); ++t) all.off.push_back(base + a.off[t]);
            all.idx.insert(all.idx.end(), a.idx.begin(), a.idx.end());
            all.pauli.insert(all.pauli.end(), a.pauli.begin(), a.pauli.end());
            all.coefs.insert(all.coefs.end(), a.coefs.begin(), a.coefs.end());
            op_off.push_back(all.off.size() - 1);
        }
        std::vector<double> out(op_off.size() - 1, 0.0);
        check(hqs_sim_get_expectation_values(h_, out.size(), op_off.data(), all.off.data(), all.idx.data(),
                                             all.pauli.data(), all.coefs.data(), ids.data(), ids.size(), out.data()));
        return out;
    }
    void apply_qubit_operator(const py::object& op, const Ids& ids) {
        const PauliArgs a = encode(op);
        check(hqs_sim_apply_qubit_operator(h_, a.off.size() - 1, a.off.data(), a.idx.data(), a.pauli.data(),
                                           a.coefs.data(), ids.data(), ids.size()));
    }
    void set_wavefunction(const std::vector<cplx>& wf, const Ids& ids) {
        check(hqs_sim_set_wavefunction(h_, reinterpret_cast<const double*>(wf.data()), wf.size(), ids.data(),
                                       ids.size()));
    }
    // --- extensions ---
    void synchronize() { check(hqs_sim_synchronize(h_)); }
    py::array_t<uint64_t> sample(uint64_t shots) {
        py::array_t<uint64_t> out((py::ssize_t)shots);
        check(hqs_sim_sample(h_, shots, out.mutable_data()));
        return out;
    }
    void move_qubits(const Ids& ids, const std::vector<int>& positions) {
        if (ids.size() != positions.size()) throw py::value_error("ids and positions differ in length");
        check(hqs_sim_move_qubits(h_, ids.data(), positions.data(), ids.size()));
    }
    void set_pass_limits(int max_tile_bits, int max_ops, int defer) {
        check(hqs_sim_set_pass_limits(h_, max_tile_bits, max_ops, defer));
    }
    py::dict stats() const {
        uint64_t s[6];
        check(hqs_sim_stats(h_, s));
        py::dict d;
        d["gates"] = s[0];
        d["runs"] = s[1];
        d["passes"] = s[2];
        d["pass_ops"] = s[3];
        d["bytes_moved"] = s[4];
        d["flushes"] = s[5];
        return d;
    }
    std::string precision() const {
        int p = 0, a = 0;
        check(hqs_sim_info(h_, &p, &a));
        return p == HQS_C64 ? "c64" : "c128";
    }
    std::string arith() const {
        int p = 0, a = 0;
        check(hqs_sim_info(h_, &p, &a));
        return a == HQS_ARITH_F64 ? "f64" : a == HQS_ARITH_DF ? "df" : a == HQS_ARITH_TC ? "tc"
               : a == HQS_ARITH_TF32 ? "tf32" : a == HQS_ARITH_TC64 ? "tc" : "f32";
    }
    void enable_pass_timing(bool on) { check(hqs_sim_set_pass_timing(h_, on ? 1 : 0)); }
    py::dict pass_timing() {
        uint64_t launches = 0, bytes = 0;
        double ms = 0;
        check(hqs_sim_pass_timing(h_, &launches, &bytes, &ms));
        py::dict d;
        d["launches"] = launches;
        d["bytes"] = bytes;
        d["ms"] = ms;
        size_t cnt = 0;
        check(hqs_sim_pass_log(h_, nullptr, 0, &cnt));
        std::vector<hqs_pass_record> rec(cnt);
        if (cnt) check(hqs_sim_pass_log(h_, rec.data(), cnt, &cnt));
        py::list log;
        for (const auto& r : rec)
            log.append(py::make_tuple(r.kernel == HQS_KERNEL_UMMA ? "umma_pass_kernel" : "pass_kernel", r.nops,
                                      r.bytes, r.ms, r.copies, r.target_mask));
        d["log"] = log;
        return d;
    }
    // Zero-copy export of the device state (position order) as a DLPack
    // capsule; owner is the Python object of this simulator.
    py::object state_dlpack(const py::object& owner) {
        void* p = nullptr;
        uint64_t amps = 0;
        int dev = 0;
        check(hqs_sim_state_view(h_, &p, &amps, &dev));
        auto* v = new StateView();
        v->shape[0] = (int64_t)amps;
        DLTensor& d = v->t.dl_tensor;
        d.data = p;
        d.device = DLDevice{2, dev};
        d.ndim = 1;
        d.dtype = DLDataType{5, (uint8_t)(precision() == "c64" ? 64 : 128), 1};
        d.shape = v->shape;
        d.strides = v->strides;
        d.byte_offset = 0;
        v->t.manager_ctx = v;
        v->t.deleter = state_view_deleter;
        v->owner = owner.ptr();
        Py_INCREF(v->owner);
        PyObject* cap = PyCapsule_New(&v->t, "dltensor", state_capsule_destructor);
        if (!cap) {
            state_view_deleter(&v->t);
            throw py::error_already_set();
        }
        return py::reinterpret_steal<py::object>(cap);
    }
    void timer_start() { check(hqs_sim_timer_start(h_)); }
    float timer_stop() {
        float ms = 0;
        check(hqs_sim_timer_stop(h_, &ms));
        return ms;
    }

private:
    hqs_sim* h_ = nullptr;
};

}  // namespace

PYBIND11_MODULE(_cppsim_mpi, m) {
    m.doc() = "GB300 state-vector engine with the interface of HiQ's _cppsim_mpi module";
    py::class_<SimulatorMPI>(m, "SimulatorMPI")
        .def(py::init<uint64_t, int64_t, int64_t, const std::string&, const std::string&>(), py::arg("seed"),
             py::arg("max_local"), py::arg("max_cluster_size"), py::arg("precision") = "", py::arg("arith") = "")
        .def("get_qubits_ids", &SimulatorMPI::get_qubits_ids)
        .def("get_local_qubits_ids", &SimulatorMPI::get_local_qubits_ids)
        .def("get_global_qubits_ids", &SimulatorMPI::get_global_qubits_ids)
        .def("set_qubits_perm", &SimulatorMPI::set_qubits_perm)
        .def("swap_qubits", &SimulatorMPI::swap_qubits)
        .def("allocate_qureg", &SimulatorMPI::allocate_qureg, py::arg("ids"), py::arg("init") = cplx(0.0, 0.0))
        .def("allocate_qubit", &SimulatorMPI::allocate_qubit)
        .def("deallocate_qubit", &SimulatorMPI::deallocate_qubit)
        .def("measure_qubits", &SimulatorMPI::measure_qubits)
        .def("apply_controlled_gate", &SimulatorMPI::apply_controlled_gate)
        .def("emulate_math", &SimulatorMPI::emulate_math)
        .def("get_amplitude", &SimulatorMPI::get_amplitude)
        .def("get_probability", &SimulatorMPI::get_probability)
        .def("run", &SimulatorMPI::run)
        .def("entropy", &SimulatorMPI::entropy)
        .def("cheat_local", &SimulatorMPI::cheat_local)
        .def("collapse_wavefunction", &SimulatorMPI::collapse_wavefunction)
        .def("get_expectation_value", &SimulatorMPI::get_expectation_value)
        .def("apply_qubit_operator", &SimulatorMPI::apply_qubit_operator)
        .def("get_expectation_values", &SimulatorMPI::get_expectation_values)
        .def("set_wavefunction", &SimulatorMPI::set_wavefunction)
        .def("emulate_time_evolution", &SimulatorMPI::emulate_time_evolution)
        .def("cheat_local_numpy", &SimulatorMPI::cheat_local_numpy)
        .def("synchronize", &SimulatorMPI::synchronize)
        .def("sample", &SimulatorMPI::sample)
        .def("move_qubits", &SimulatorMPI::move_qubits)
        .def("set_pass_limits", &SimulatorMPI::set_pass_limits, py::arg("max_tile_bits") = 0, py::arg("max_ops") = 0,
             py::arg("defer") = 0)
        .def("stats", &SimulatorMPI::stats)
        .def("enable_pass_timing", &SimulatorMPI::enable_pass_timing)
        .def("pass_timing", &SimulatorMPI::pass_timing)
        .def("state_dlpack", [](py::object self) { return self.cast<SimulatorMPI&>().state_dlpack(self); })
        .def("timer_start", &SimulatorMPI::timer_start)
        .def("timer_stop", &SimulatorMPI::timer_stop)
        .def_property_readonly("precision", &SimulatorMPI::precision)
        .def_property_readonly("arith", &SimulatorMPI::arith);
}
