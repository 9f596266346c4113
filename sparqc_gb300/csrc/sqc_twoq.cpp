// Two-qubit gates as sequences of the engine's own gates (no counterpart in the reference,
// whose gate set is eight uncontrolled single-qubit gates, emulator/include/circuit.h:45-83).
//
// A two-qubit gate acts on the four basis states of qubits (a, b), indexed i_a + 2 i_b. Rather
// than a fifth pass layout, every two-qubit gate becomes a short run of single-qubit and
// controlled gates, which the planner resolves and fuses into the usual passes like any other
// gates (a gate on two qubits >= 4 becomes one quad pass).
//
// * General unitary (decompose_2q): the textbook reduction to two-level unitaries (Nielsen and
//   Chuang, "Quantum Computation and Quantum Information", sec. 4.5.1). Left-multiplying U by
//   Givens rotations G_1..G_6, each acting on two basis states that differ in one qubit, clears
//   U's entries below the diagonal column by column; each rotation is chosen in SU(2) with a
//   real positive pivot, so what remains is diag(1, 1, 1, det U) up to rounding. Then
//   U = G_1^+ ... G_6^+ diag(1, 1, 1, det U). A two-level unitary on states that differ in qubit
//   t while the other qubit o equals v is a gate on t controlled by o (by NOT o when v = 0: X on o
//   before and after, a relabelling of the keys on the host); its SU(2) matrix is written as
//   e^{i gamma} U3(theta, phi, lambda), a U gate and a Phase(gamma) on o under the same condition.
// * Named forms with exact short decompositions (permutations and exact phases stay exact):
//   RZZ(theta) = exp(-i theta/2 Z_a Z_b): Rz(theta) on b where a = 0, Rz(-theta) on b where a = 1;
//   iSWAP: CX(a->b) S_b CX(b->a) CX(a->b); fSim(theta, phi): CX(a->b), Rx(2 theta) on a controlled
//   by b, CX(a->b), then Phase(-phi) on b controlled by a; CSWAP (Fredkin): CX(b->a) CCX(c, a->b)
//   CX(b->a).
// User controls are added to every gate that acts on amplitudes; the X/CX pairs around them
// cancel where the controls do not hold.
#include <cmath>
#include <complex>
#include <vector>

#include "sqc_twoq.h"

namespace sqc {
namespace {

using cd = std::complex<double>;

sqc_gate gate(uint32_t kind, uint32_t t, uint64_t ctrl, double th = 0.0, double ph = 0.0, double la = 0.0) {
    sqc_gate g;
    g.kind = kind;
    g.target = t;
    g.controls = ctrl;
    g.theta = th;
    g.phi = ph;
    g.lambda = la;
    return g;
}

// Append W (2x2 unitary, rows/columns: qubit t = 0, 1) acting where qubit o == v and the
// controls C hold: e^{i gamma} U3(theta, phi, lambda) as a U gate on t and a Phase on o.
void two_level(std::vector<sqc_gate>& out, const cd W[2][2], uint32_t t, uint32_t o, int v, uint64_t C) {
    const cd alpha = W[0][0], beta = W[1][0];
    const double ma = std::abs(alpha), mb = std::abs(beta);
    if (mb < 1e-300 && std::abs(alpha - cd(1.0, 0.0)) < 1e-300 && std::abs(W[1][1] - cd(1.0, 0.0)) < 1e-300)
        return;   // identity
    // W = e^{i gamma} [[cos, -e^{i lambda} sin], [e^{i phi} sin, e^{i(phi+lambda)} cos]], det W = e^{2 i gamma + i(phi+lambda)}
    const double theta = 2.0 * std::atan2(mb, ma);
    double gamma, phi, lam;
    if (ma > 0.0) {
        gamma = std::arg(alpha);
        phi = mb > 0.0 ? std::arg(beta) - gamma : 0.0;
        lam = std::arg(W[1][1]) - gamma - phi;
    } else {   // W = [[0, w01], [beta, 0]]
        gamma = 0.0;
        phi = std::arg(beta);
        lam = std::arg(-W[0][1]);
    }
    const uint64_t ob = 1ULL << o;
    if (!v) out.push_back(gate(SQC_X, o, 0));
    out.push_back(gate(SQC_U, t, C | ob, theta, phi, lam));
    if (gamma != 0.0) out.push_back(gate(SQC_PHASE, o, C, gamma));
    if (!v) out.push_back(gate(SQC_X, o, 0));
}

// Gates that apply the 4x4 unitary u (row-major (re, im) pairs, index i_a + 2 i_b) to qubits a, b
// under controls C. Returns nullptr, or the reason u was rejected.
const char* decompose_2q(uint32_t a, uint32_t b, uint64_t C, const double* u, std::vector<sqc_gate>& out) {
    cd M[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) M[r][c] = cd(u[2 * (4 * r + c)], u[2 * (4 * r + c) + 1]);
    // unitarity to 1e-9
    for (int r = 0; r < 4; ++r)
        for (int s = 0; s < 4; ++s) {
            cd acc = 0.0;
            for (int c = 0; c < 4; ++c) acc += M[r][c] * std::conj(M[s][c]);
            if (std::abs(acc - (r == s ? cd(1.0) : cd(0.0))) > 1e-9) return "the matrix is not unitary";
        }
    // basis index -> (bit of a, bit of b); the qubit two states differ in, and the other one's value
    struct Step { int col, p, q; bool keep_p; };
    // column by column; each pair differs in one qubit: (2,3) and (0,1) in a, (0,2) and (1,3) in b
    const Step steps[6] = {{0, 2, 3, true}, {0, 0, 2, true}, {0, 0, 1, true},
                           {1, 2, 3, false}, {1, 1, 3, true}, {2, 2, 3, true}};
    cd G[6][2][2];
    for (int k = 0; k < 6; ++k) {
        const Step& s = steps[k];
        const cd x = M[s.p][s.col], y = M[s.q][s.col];
        const double r = std::hypot(std::abs(x), std::abs(y));
        cd g[2][2];
        if (r == 0.0) {
            g[0][0] = 1.0; g[0][1] = 0.0; g[1][0] = 0.0; g[1][1] = 1.0;
        } else if (s.keep_p) {   // new p = r, new q = 0
            g[0][0] = std::conj(x) / r; g[0][1] = std::conj(y) / r;
            g[1][0] = -y / r;           g[1][1] = x / r;
        } else {                 // new p = 0, new q = r
            g[0][0] = y / r;            g[0][1] = -x / r;
            g[1][0] = std::conj(x) / r; g[1][1] = std::conj(y) / r;
        }
        for (int c = 0; c < 4; ++c) {
            const cd mp = M[s.p][c], mq = M[s.q][c];
            M[s.p][c] = g[0][0] * mp + g[0][1] * mq;
            M[s.q][c] = g[1][0] * mp + g[1][1] * mq;
        }
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) G[k][i][j] = g[i][j];
    }
    // U = G_1^+ ... G_6^+ D, D = diag(1, 1, 1, d3): applied to the state in the order D, G_6^+, ..., G_1^+
    const cd d3 = M[3][3] / std::abs(M[3][3]);
    const double ph = std::arg(d3);
    if (ph != 0.0) out.push_back(gate(SQC_PHASE, b, C | (1ULL << a), ph));
    for (int k = 5; k >= 0; --k) {
        const Step& s = steps[k];
        cd W[2][2];   // G^+ on (p, q)
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j) W[i][j] = std::conj(G[k][j][i]);
        const int diff = s.p ^ s.q;                 // 1: the states differ in a, 2: in b
        const uint32_t t = diff == 1 ? a : b, o = diff == 1 ? b : a;
        const int v = diff == 1 ? (s.p >> 1) & 1 : s.p & 1;   // the other qubit's value on both states
        two_level(out, W, t, o, v, C);
    }
    return nullptr;
}

void rzz_2q(uint32_t a, uint32_t b, uint64_t C, double theta, std::vector<sqc_gate>& out) {
    const uint64_t am = 1ULL << a;
    out.push_back(gate(SQC_X, a, 0));
    out.push_back(gate(SQC_RZ, b, C | am, theta));
    out.push_back(gate(SQC_X, a, 0));
    out.push_back(gate(SQC_RZ, b, C | am, -theta));
}

void iswap_2q(uint32_t a, uint32_t b, uint64_t C, std::vector<sqc_gate>& out) {
    out.push_back(gate(SQC_X, b, C | (1ULL << a)));
    out.push_back(gate(SQC_S, b, C));
    out.push_back(gate(SQC_X, a, C | (1ULL << b)));
    out.push_back(gate(SQC_X, b, C | (1ULL << a)));
}

void fsim_2q(uint32_t a, uint32_t b, uint64_t C, double theta, double phi, std::vector<sqc_gate>& out) {
    out.push_back(gate(SQC_X, b, C | (1ULL << a)));
    out.push_back(gate(SQC_RX, a, C | (1ULL << b), 2.0 * theta));
    out.push_back(gate(SQC_X, b, C | (1ULL << a)));
    out.push_back(gate(SQC_PHASE, b, C | (1ULL << a), -phi));
}

void cswap_2q(uint32_t c, uint32_t a, uint32_t b, uint64_t C, std::vector<sqc_gate>& out) {
    out.push_back(gate(SQC_X, a, C | (1ULL << b)));
    out.push_back(gate(SQC_X, b, C | (1ULL << c) | (1ULL << a)));
    out.push_back(gate(SQC_X, a, C | (1ULL << b)));
}

}  // namespace

int twoq_sequence(uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta, double phi,
                  const double* u, std::vector<sqc_gate>& out) {
    if (a > 63 || b > 63 || a == b) return SQC_ERR_ARG;
    uint64_t used = (1ULL << a) | (1ULL << b);
    if (form == SQC_2Q_CSWAP) {
        if (c > 63 || c == a || c == b) return SQC_ERR_ARG;
        used |= 1ULL << c;
    }
    if (controls & used) return SQC_ERR_ARG;
    switch (form) {
    case SQC_2Q_UNITARY:
        if (!u || decompose_2q(a, b, controls, u, out)) return SQC_ERR_ARG;
        return SQC_OK;
    case SQC_2Q_RZZ: rzz_2q(a, b, controls, theta, out); return SQC_OK;
    case SQC_2Q_ISWAP: iswap_2q(a, b, controls, out); return SQC_OK;
    case SQC_2Q_FSIM: fsim_2q(a, b, controls, theta, phi, out); return SQC_OK;
    case SQC_2Q_CSWAP: cswap_2q(c, a, b, controls, out); return SQC_OK;
    case SQC_2Q_SWAP:
        out.push_back(gate(SQC_X, a, controls | (1ULL << b)));
        out.push_back(gate(SQC_X, b, controls | (1ULL << a)));
        out.push_back(gate(SQC_X, a, controls | (1ULL << b)));
        return SQC_OK;
    default: return SQC_ERR_ARG;
    }
}

}  // namespace sqc
