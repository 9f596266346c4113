// Two-qubit gates as sequences of the engine's own gates (sqc_twoq.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/sparqc.h"

namespace sqc {

// The gates of one two-qubit gate of the given form (SQC_2Q_*), appended to out. Returns SQC_OK,
// or SQC_ERR_ARG for a bad form, equal or out-of-range qubits, controls on a target, or a
// matrix that is not unitary.
int twoq_sequence(uint32_t form, uint32_t a, uint32_t b, uint32_t c, uint64_t controls, double theta, double phi,
                  const double* u, std::vector<sqc_gate>& out);

}  // namespace sqc
