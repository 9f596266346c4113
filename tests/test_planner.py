"""Host-side planning and memory bookkeeping, on the CPU (no GPU needed).

A small C++ program is compiled against sparqc_gb300/csrc/sqc_plan.{h,cpp} and sqc_pool.h
and run here: it checks how gates are resolved against the known key bits, how descriptor
sequences are cut into passes with one or two cross-group qubits, the group bound that sizes
batch slices, and the first-fit pool of the serving loop.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sparqc_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")

PROGRAM = r'''
#include <cstdio>
#include <cstring>
#include <vector>
#include "sqc_plan.h"
#include "sqc_pool.h"
using namespace sqc;

static int fails = 0;
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); ++fails; } } while (0)

static sqc_gate g(uint32_t kind, uint32_t t, uint64_t ctrl = 0, double th = 0.3) {
    sqc_gate x; std::memset(&x, 0, sizeof x);
    x.kind = kind; x.target = t; x.controls = ctrl; x.theta = th;
    return x;
}

struct P { size_t g0, g1; uint32_t nx, q1, q2, q3; bool fixed; };

static std::vector<P> split(const std::vector<GateDesc>& d, uint32_t max_nx, size_t max_run = 64) {
    std::vector<P> out;
    split_passes(d.data(), d.size(), max_run, max_nx,
                 [&](size_t a, size_t b, uint32_t nx, uint32_t q1, uint32_t q2, uint32_t q3, bool f) {
        out.push_back(P{a, b, nx, q1, q2, q3, f});
    });
    return out;
}

int main() {
    // resolution against known bits: |0..0> knows every bit
    Planner p;
    GateDesc d;
    CHECK(!plan_gate(p, g(KX, 7), &d));                 // uncontrolled X: frame flip
    CHECK(p.frame == (1ULL << 7) && p.kval == (1ULL << 7));
    CHECK(!plan_gate(p, g(KH, 3, 1ULL << 9), &d));       // control 9 known 0: identity
    CHECK(p.credit == 2);
    CHECK(plan_gate(p, g(KH, 3, 1ULL << 7), &d));        // control 7 known 1: dropped, H acts
    CHECK(d.ctrl == 0 && d.kind == KH);
    CHECK((p.kmask & (1ULL << 3)) == 0);                 // bit 3 now varies
    CHECK(!plan_gate(p, g(KZ, 5), &d));                  // Z on a known-0 bit: identity
    CHECK(plan_gate(p, g(KY, 6), &d) && d.kind == KYPH); // uncontrolled Y: relabel + diagonal
    CHECK(group_bound(p, 20) == 1);                      // only bit 3 varies: one group
    CHECK(plan_gate(p, g(KRX, 12), &d));
    CHECK(plan_gate(p, g(KX, 13, 1ULL << 12), &d));      // controlled by a varying bit: on the device
    CHECK(group_bound(p, 20) == 4);                      // bits 12, 13 vary
    CHECK(std::strcmp(check_gate(g(KH, 20), 20), "target qubit out of range") == 0);
    CHECK(check_gate(g(KH, 3, 1ULL << 3), 20) != nullptr);
    CHECK(check_gate(g(KU, 19, 1ULL << 18), 20) == nullptr);

    // pass split: gates on qubits 5, 6, 5, 7 with streamable gates in between
    std::vector<GateDesc> s;
    Planner q;
    q.kmask = 0; q.kval = 0;                            // nothing known: every gate stays
    for (auto gg : {g(KH, 5), g(KZ, 9), g(KH, 2), g(KRY, 6), g(KH, 5), g(KRX, 7), g(KT, 7), g(KH, 1)}) {
        GateDesc x; CHECK(plan_gate(q, gg, &x)); s.push_back(x);
    }
    auto one = split(s, 1);
    CHECK(one.size() == 4);
    CHECK(one[0].g0 == 0 && one[0].g1 == 3 && one[0].nx == 1 && one[0].q1 == 5);
    CHECK(one[1].g0 == 3 && one[1].g1 == 4 && one[1].q1 == 6);
    CHECK(one[2].g0 == 4 && one[2].g1 == 5 && one[2].q1 == 5);
    CHECK(one[3].g0 == 5 && one[3].g1 == 8 && one[3].q1 == 7 && one[3].nx == 1);
    auto two = split(s, 2);
    CHECK(two.size() == 2);
    CHECK(two[0].g0 == 0 && two[0].g1 == 5 && two[0].nx == 2 && two[0].q1 == 5 && two[0].q2 == 6);
    CHECK(two[1].g0 == 5 && two[1].g1 == 8 && two[1].nx == 1 && two[1].q1 == 7 && two[1].q2 == kNoQubit);
    auto capped = split(s, 2, 2);                       // at most 2 gates per pass
    CHECK(capped.size() == 4);
    auto three = split(s, 3);                           // qubits 5, 6, 7 in one pass
    CHECK(three.size() == 1);
    CHECK(three[0].nx == 3 && three[0].q1 == 5 && three[0].q2 == 6 && three[0].q3 == 7);
    CHECK(split(s, 4).size() == 1);                     // more than three is three
    {   // encoding: q1 and q3 pair lane-local slots, q2 and qubits 0..3 shuffle
        std::vector<GateDesc> e = s;
        encode_pass(e.data(), 0, e.size(), 5, 7);
        CHECK((e[0].flip & kOpPair) && !(e[0].flip & kOpPair3));               // H 5
        CHECK((e[3].flip & kOpShfl) && ((e[3].flip >> kOpOffShift) & 7u) == 4); // Ry 6: other half
        CHECK((e[5].flip & kOpPair3) && !(e[5].flip & kOpPair));               // Rx 7
        CHECK((e[2].flip & kOpShfl) && ((e[2].flip >> kOpOffShift) & 7u) == 2); // H 2: lane ^ 4
        CHECK(!(e[1].flip & (kOpPair | kOpPair3 | kOpShfl)));                 // Z 9: lane-local
    }
    std::vector<GateDesc> diag;
    for (auto gg : {g(KZ, 30), g(KRZ, 40), g(KT, 2)}) { GateDesc x; CHECK(plan_gate(q, gg, &x)); diag.push_back(x); }
    auto dd = split(diag, 2);
    CHECK(dd.size() == 1 && dd[0].nx == 0 && dd[0].fixed);

    // first-fit pool with coalescing
    RangePool pool;
    pool.reset(1 << 20, 256);
    size_t a = pool.alloc(1000), b = pool.alloc(5000), c = pool.alloc(300);
    CHECK(a == 0 && b == 1024 && c == 1024 + 5120);
    CHECK(pool.used() == 1024 + 5120 + 512);
    pool.release(b, 5000);
    CHECK(pool.alloc(6000) == 1024 + 5120 + 512);        // does not fit the hole: after c
    size_t h = pool.alloc(4000);
    CHECK(h == 1024);                                    // fits the hole
    pool.release(a, 1000); pool.release(h, 4000); pool.release(c, 300);
    pool.release(1024 + 5120 + 512, 6000);
    CHECK(pool.used() == 0 && pool.largest_free() == (1u << 20));
    CHECK(pool.alloc(2u << 20) == SIZE_MAX);

    // scheduling: H4 H5 H6 H4 H5 with two cross-group qubits per pass takes three passes in
    // order; H4 and H5 share no qubit with H6 and move ahead of it: two passes
    {
        std::vector<sqc_gate> gs = {g(KH, 4), g(KH, 5), g(KH, 6), g(KH, 4), g(KH, 5)};
        uint32_t perm[5];
        schedule_gates(gs.data(), gs.size(), 2, 64, 256, perm);
        const uint32_t want[5] = {0, 1, 3, 4, 2};
        for (int i = 0; i < 5; ++i) CHECK(perm[i] == want[i]);
        auto passes = [&](const std::vector<sqc_gate>& v) {
            Planner q;
            std::vector<GateDesc> dv;
            for (const sqc_gate& x : v) { GateDesc y; if (plan_gate(q, x, &y)) dv.push_back(y); }
            return split(dv, 2).size();
        };
        std::vector<sqc_gate> s;
        for (int i = 0; i < 5; ++i) s.push_back(gs[perm[i]]);
        CHECK(passes(gs) == 3 && passes(s) == 2);
        // one cross-group qubit per pass: Rz(4) moves ahead of H(5) and Rz(5) (neither changes
        // a qubit the other touches); Rz(5) stays behind H(5), which changes its qubit
        std::vector<sqc_gate> h = {g(KH, 4), g(KH, 5), g(KRZ, 5), g(KRZ, 4)};
        uint32_t ph[4];
        schedule_gates(h.data(), h.size(), 1, 64, 256, ph);
        const uint32_t wh[4] = {0, 3, 1, 2};
        for (int i = 0; i < 4; ++i) CHECK(ph[i] == wh[i]);
        // the pass's qubits by trial: on (5, 6) the first pass takes H5, H6, CX(6 -> 5), Rz5
        // and Rz7, none of which touches qubit 4; on the first-use choice (4, 5) it would take
        // only H4, H5 and Rz7 (H6, left behind, changes the CX's control)
        std::vector<sqc_gate> k = {g(KH, 4), g(KH, 5), g(KH, 6), g(KX, 5, 1ULL << 6), g(KRZ, 5), g(KRZ, 7)};
        uint32_t pk[6];
        schedule_gates(k.data(), k.size(), 2, 64, 256, pk);
        const uint32_t wk[6] = {1, 2, 3, 4, 5, 0};
        for (int i = 0; i < 6; ++i) CHECK(pk[i] == wk[i]);
    }
    // every gate plans the same in the scheduled order as in the given one (same resolution on
    // the host, same descriptor), and the planner ends in the same state: random circuits of
    // every gate kind, up to three controls, on 12, 40 and 64 qubits
    {
        unsigned long long rs = 0x9E3779B97F4A7C15ULL;
        auto rnd = [&]() { rs = rs * 6364136223846793005ULL + 1442695040888963407ULL; return rs >> 33; };
        const uint32_t kinds[] = {KX, KY, KZ, KH, KPHASE, KRZ, KRX, KRY, KS, KSDG, KT, KTDG, KU};
        int checked = 0, moved = 0;
        for (uint32_t nq : {12u, 40u, 64u}) {
            for (int rep = 0; rep < 4; ++rep) {
                std::vector<sqc_gate> gs;
                const uint32_t kq = nq < 16 ? nq : 16;   // branching gates stay below qubit kq
                for (uint32_t q = 0; q < kq; ++q) gs.push_back(g(KH, q));
                for (int i = 0; i < 400; ++i) {
                    const uint32_t kind = kinds[rnd() % 13];
                    const bool branch = kind == KH || kind == KRX || kind == KRY || kind == KU;
                    const uint32_t t = (uint32_t)(branch ? rnd() % kq : rnd() % nq);
                    uint64_t ctl = 0;
                    for (uint32_t c = 0, nc = (uint32_t)(rnd() % 4); c < nc; ++c) {
                        const uint32_t q = (uint32_t)(rnd() % nq);
                        if (q != t) ctl |= 1ULL << q;
                    }
                    sqc_gate x = g(kind, t, ctl, 0.1 + 0.01 * (double)(rnd() % 500));
                    x.phi = 0.3; x.lambda = 0.7;
                    gs.push_back(x);
                }
                for (uint32_t mx = 1; mx <= 3; ++mx) {
                    std::vector<uint32_t> perm(gs.size());
                    schedule_gates(gs.data(), gs.size(), mx, 64, 256, perm.data());
                    std::vector<char> seen(gs.size(), 0);
                    bool ok = true;
                    for (uint32_t i : perm) { ok = ok && i < gs.size() && !seen[i]; if (i < gs.size()) seen[i] = 1; }
                    CHECK(ok);
                    if (!ok) continue;
                    Planner a, b;
                    std::vector<GateDesc> da(gs.size()), db(gs.size());
                    std::vector<char> ra(gs.size()), rb(gs.size());
                    for (size_t i = 0; i < gs.size(); ++i) { std::memset(&da[i], 0, sizeof(GateDesc)); ra[i] = plan_gate(a, gs[i], &da[i]); }
                    for (size_t j = 0; j < gs.size(); ++j) {
                        const uint32_t i = perm[j];
                        std::memset(&db[i], 0, sizeof(GateDesc));
                        rb[i] = plan_gate(b, gs[i], &db[i]);
                        moved += i != j;
                    }
                    for (size_t i = 0; i < gs.size(); ++i) {
                        da[i].pad = db[i].pad = 0;   // the credit of host-resolved gates before it
                        CHECK(ra[i] == rb[i]);
                        CHECK(!ra[i] || std::memcmp(&da[i], &db[i], sizeof(GateDesc)) == 0);
                        ++checked;
                    }
                    CHECK(a.frame == b.frame && a.kmask == b.kmask && a.kval == b.kval);
                }
            }
        }
        CHECK(checked > 10000 && moved > 1000);
    }

    std::printf("fails=%d\n", fails);
    return fails ? 1 : 0;
}
'''


def test_planner_and_pool(tmp_path):
    src = tmp_path / "planner.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "planner"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", INCLUDE, "-I", CSRC, str(src),
                        os.path.join(CSRC, "sqc_plan.cpp"), "-o", str(exe)], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail(r.stderr)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "fails=0" in out.stdout
