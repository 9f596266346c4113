/*
 * sparqc_circuit.hpp -- C++ drop-in for the reference's circuit API.
 *
 * Keeps the names, arguments and error behaviour of ivanNovikau/SparQC's Circuit__
 * (emulator/include/circuit.h:12-265) and hash_table_parameters
 * (emulator/include/sim_parameters_types.h:133-145) over the C ABI in sparqc.h:
 *   Circuit__ oc(nq, hp);  oc.h(t); oc.rx(t, par); ...  oc.print_raw_data();
 * Errors throw std::string, as the reference does (caught at emulator/src/main.cu:374).
 * Additions: s/sdg/t/tdg/u, controlled forms taking a control list, apply(gates),
 * get_state (key-sorted arrays), nnz, norm2, sync.
 */
#ifndef SPARQC_CIRCUIT_HPP
#define SPARQC_CIRCUIT_HPP

#include <cstdint>
#include <cstdio>
#include <initializer_list>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "sparqc.h"

/* Same fields as the reference; N_subtables and log2_N_bucket_spots are accepted and ignored
 * (buckets always hold 16 keys). The added fields have defaults. */
struct hash_table_parameters {
    uint32_t N_devices = 1;
    double coef_gpu_memory_reserve = 0.01;
    uint32_t N_subtables = 1;
    uint32_t log2_N_bucket_spots = 4;
    uint32_t precision = SQC_FP64;      /* added: SQC_FP64 or SQC_FP32 amplitudes */
    double prune_threshold = 1e-14;     /* added */
    double load_factor = 0.5;           /* added */
};

struct TComplex {
    double r;
    double i;
};

class Circuit__ {
public:
    Circuit__(uint32_t nq, const hash_table_parameters& hp) : nq_(nq) {
        sqc_hash_table_parameters p;
        p.N_devices = hp.N_devices;
        p.coef_gpu_memory_reserve = hp.coef_gpu_memory_reserve;
        p.N_subtables = hp.N_subtables;
        p.log2_N_bucket_spots = hp.log2_N_bucket_spots;
        sqc_options o;
        sqc_default_options(&o);
        o.precision = hp.precision;
        o.prune_threshold = hp.prune_threshold;
        o.load_factor = hp.load_factor;
        check(sqc_create(nq, &p, &o, &st_), "Circuit__");
    }
    ~Circuit__() { sqc_destroy(st_); }
    Circuit__(const Circuit__&) = delete;
    Circuit__& operator=(const Circuit__&) = delete;

    /* reference gates (emulator/include/circuit.h:45-83) */
    void x(uint32_t t) { gate(SQC_X, t); }
    void y(uint32_t t) { gate(SQC_Y, t); }
    void z(uint32_t t) { gate(SQC_Z, t); }
    void h(uint32_t t) { gate(SQC_H, t); }
    void phase(uint32_t t, double par) { gate(SQC_PHASE, t, par); }
    void rz(uint32_t t, double par) { gate(SQC_RZ, t, par); }
    void rx(uint32_t t, double par) { gate(SQC_RX, t, par); }
    void ry(uint32_t t, double par) { gate(SQC_RY, t, par); }

    /* additions */
    void s(uint32_t t) { gate(SQC_S, t); }
    void sdg(uint32_t t) { gate(SQC_SDG, t); }
    void t(uint32_t q) { gate(SQC_T, q); }
    void tdg(uint32_t q) { gate(SQC_TDG, q); }
    void u(uint32_t t, double theta, double phi, double lambda) { gate(SQC_U, t, theta, 0, phi, lambda); }
    /* any gate kind with a list of control qubits, e.g. oc.controlled(SQC_X, 5, {0, 1}) */
    void controlled(uint32_t kind, uint32_t t, std::initializer_list<uint32_t> controls, double theta = 0.0,
                    double phi = 0.0, double lambda = 0.0) {
        uint64_t m = 0;
        for (uint32_t c : controls) m |= uint64_t(1) << c;
        gate(kind, t, theta, m, phi, lambda);
    }
    /* two-qubit gates (sqc_apply_twoq); u: 4x4 row-major (re, im) pairs, index i_a + 2 i_b */
    void unitary2(uint32_t a, uint32_t b, const double* u, uint64_t controls = 0) {
        check(sqc_apply_twoq(st_, SQC_2Q_UNITARY, a, b, 0, controls, 0.0, 0.0, u), "unitary2");
    }
    void rzz(uint32_t a, uint32_t b, double theta) {
        check(sqc_apply_twoq(st_, SQC_2Q_RZZ, a, b, 0, 0, theta, 0.0, nullptr), "rzz");
    }
    void iswap(uint32_t a, uint32_t b) { check(sqc_apply_twoq(st_, SQC_2Q_ISWAP, a, b, 0, 0, 0.0, 0.0, nullptr), "iswap"); }
    void fsim(uint32_t a, uint32_t b, double theta, double phi) {
        check(sqc_apply_twoq(st_, SQC_2Q_FSIM, a, b, 0, 0, theta, phi, nullptr), "fsim");
    }
    void cswap(uint32_t c, uint32_t a, uint32_t b) {
        check(sqc_apply_twoq(st_, SQC_2Q_CSWAP, a, b, c, 0, 0.0, 0.0, nullptr), "cswap");
    }
    void swap(uint32_t a, uint32_t b) { check(sqc_apply_twoq(st_, SQC_2Q_SWAP, a, b, 0, 0, 0.0, 0.0, nullptr), "swap"); }
    void apply(const std::vector<sqc_gate>& gates) {
        check(sqc_apply_gates(st_, gates.data(), gates.size()), "apply");
    }

    void set_zero_quantum_state() { check(sqc_set_zero_state(st_), "set_zero_quantum_state"); }
    void sync() { check(sqc_sync(st_), "sync"); }
    uint64_t nnz() {
        uint64_t n = 0;
        check(sqc_nnz(st_, &n), "nnz");
        return n;
    }
    double norm2() {
        double v = 0.0;
        check(sqc_norm2(st_, &v), "norm2");
        return v;
    }

    /* key-sorted readout of the non-negligible entries, as the reference's readout filters them */
    void get_state(std::vector<uint64_t>& keys, std::vector<double>& re, std::vector<double>& im,
                   bool drop_negligible = true) {
        uint64_t n = nnz();
        keys.resize(n);
        re.resize(n);
        im.resize(n);
        uint32_t flags = SQC_READ_SORTED | (drop_negligible ? SQC_READ_DROP_NEGLIGIBLE : 0u);
        check(sqc_get_state(st_, keys.data(), re.data(), im.data(), n, &n, flags), "get_state");
        keys.resize(n);
        re.resize(n);
        im.resize(n);
    }

    /* reference readout: unordered map of non-negligible entries (emulator/include/circuit.h:111-126) */
    const std::unordered_map<uint64_t, TComplex>& form_unordered_statevector() {
        std::vector<uint64_t> k;
        std::vector<double> r, i;
        get_state(k, r, i, true);
        vv_.clear();
        vv_.reserve(k.size());
        for (size_t n = 0; n < k.size(); ++n) vv_[k[n]] = TComplex{r[n], i[n]};
        return vv_;
    }

    /* Key-ordered non-negligible entries matching a per-qubit pattern, as get_state_full selects
     * them (emulator/include/circuit.h:206-253): state_to_choose[q] is -1 (any), 0 or 1; an
     * empty pattern selects everything. The selection and the ordering run on the GPU. */
    std::map<uint64_t, TComplex> get_state_full(const std::vector<short>& state_to_choose = {}) {
        uint64_t mask = 0, value = 0;
        for (size_t q = 0; q < state_to_choose.size() && q < 64; ++q) {
            if (state_to_choose[q] < 0) continue;
            mask |= uint64_t(1) << q;
            if (state_to_choose[q]) value |= uint64_t(1) << q;
        }
        uint64_t n = nnz();
        std::vector<uint64_t> k(n);
        std::vector<double> r(n), i(n);
        check(sqc_get_state_where(st_, mask, value, k.data(), r.data(), i.data(), n, &n,
                                  SQC_READ_SORTED | SQC_READ_DROP_NEGLIGIBLE),
              "get_state_full");
        std::map<uint64_t, TComplex> out;
        for (uint64_t m = 0; m < n; ++m) out.emplace_hint(out.end(), k[m], TComplex{r[m], i[m]});
        return out;
    }

    /* additions: probability of a pattern, measurement of one qubit with collapse, sampling */
    double probability(uint64_t mask, uint64_t value) {
        double p = 0.0;
        check(sqc_probability(st_, mask, value, &p), "probability");
        return p;
    }
    int measure(uint32_t q, double u, double* p1 = nullptr) {
        int out = 0;
        check(sqc_measure(st_, q, u, &out, p1), "measure");
        return out;
    }
    std::vector<uint64_t> sample(uint64_t shots, uint64_t seed = 0) {
        std::vector<uint64_t> k(shots);
        check(sqc_sample(st_, shots, seed, k.data()), "sample");
        return k;
    }

    /* prints "key: re + imj" per nonzero, as print_raw_data does (emulator/include/circuit.h:88-92) */
    void print_raw_data() {
        std::vector<uint64_t> k;
        std::vector<double> r, i;
        get_state(k, r, i, true);
        for (size_t n = 0; n < k.size(); ++n)
            std::printf("%llu: \t%.3e + %.3ej\n", (unsigned long long)k[n], r[n], i[n]);
    }
    void print_full_statevector() { print_raw_data(); }

    sqc_state* handle() { return st_; }
    uint32_t nq() const { return nq_; }

private:
    void gate(uint32_t kind, uint32_t t, double theta = 0.0, uint64_t controls = 0, double phi = 0.0,
              double lambda = 0.0) {
        sqc_gate g;
        g.kind = kind;
        g.target = t;
        g.controls = controls;
        g.theta = theta;
        g.phi = phi;
        g.lambda = lambda;
        check(sqc_apply_gates(st_, &g, 1), "gate");
    }
    void check(int rc, const char* what) {
        if (rc != SQC_OK) {
            std::string msg = std::string(what) + ": " + sqc_status_string(rc);
            if (st_) {
                const char* e = sqc_last_error(st_);
                if (e && *e) msg += std::string(" (") + e + ")";
            }
            throw msg;
        }
    }

    uint32_t nq_;
    sqc_state* st_ = nullptr;
    std::unordered_map<uint64_t, TComplex> vv_;
};

#endif /* SPARQC_CIRCUIT_HPP */
