// Host emulation of the reference's FC gate kernels -- TEST INFRASTRUCTURE ONLY.
//
// This file compiles the reference's own device headers where they lie
// (emulator/device/device_table_FC.cuh, device_data.cuh, table.cuh and the headers they
// include) with g++, so that the reference's gate arithmetic, pair rule and pruning run on
// the CPU. Nothing of the reference is copied: the headers are included from the reference
// tree by the build recipe in build.py. With a host compiler the CUDA qualifiers
// (__global__, __device__, __constant__) are ignored attributes, so every kernel becomes a
// plain function; this file supplies the launch indices and runs each "launch" serially
// over its grid. Kernels on this path use no shared memory and no barriers, so a serial
// order is one valid interleaving of the threads.
//
// Emulated call sequence, following emulator/device/table_manager.cuh:
//   init     -> device_init_arrays + FC__::set_to_zero_quantum_state   (:299-308)
//   gate     -> FC__::gate_sq<sel>(t) or FC__::gate_sq_par<sel>(t, par'), then
//               device_zero_arrays, then ++counter                       (:311-340)
//               with par' = par for Phase and par/2 for Rz, Rx, Ry      (:333-336)
//   readout  -> the current half of the KV array, dropping negligible values (table.cuh:47-75)
// The grid-stride loops make the result independent of the grid size except where the
// reference itself races. Two of its races are handled here:
//   - device_zero_arrays lets global thread 0 overwrite N_ while other threads still use it
//     as their loop bound (device_data.cuh:72-80); thread 0 is run last, which is the
//     intended behaviour.
//   - gate_sq_par writes the skip-path address-book entry even for Rx/Ry
//     (device_table_FC.cuh:190-193), where it collides with the atomic appends of
//     update_ah_sup. That corrupts the address book whenever an Rx/Ry pair has both members
//     present; refemu_gate reports such a gate with return code 1 so callers can avoid or
//     flag it. The emulation still runs the reference code unchanged.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <algorithm>
#include <vector>
#include <iostream>
#include <sstream>
#include <fstream>
#include <iomanip>
#include <memory>
#include <string>
#include <stdexcept>
#include <filesystem>
#include <ctime>
#include <list>
#include <map>
#include <unordered_map>
#include <iterator>
#include <limits>
#include <chrono>
#include <cstdarg>
#include <numeric>
#include <unistd.h>
#include <cuda_runtime_api.h>

static uint3 emu_threadIdx, emu_blockIdx;
static dim3 emu_blockDim, emu_gridDim;
#define threadIdx emu_threadIdx
#define blockIdx emu_blockIdx
#define blockDim emu_blockDim
#define gridDim emu_gridDim

static inline uint32_t atomicAdd(uint32_t* p, uint32_t v) { uint32_t o = *p; *p = o + v; return o; }
static inline uint3 emu_idx(uint32_t x) { uint3 u; u.x = x; u.y = 0; u.z = 0; return u; }

// The kernels print progress lines on every gate; a host run keeps them quiet.
#define printf(...) ((void)0)
#include "device_table_FC.cuh"
#undef printf

namespace {

constexpr uint32_t kThreads = N_THREADS;   // 128, emulator/include/sim_parameters_types.h:49
constexpr uint32_t kMaxBlocks = 64;        // any grid gives the same result (grid-stride loops)

std::vector<KV> g_kv;
std::vector<thash> g_ah;
uint32_t g_counter = 0;
uint32_t g_blocks = 1;
bool g_live = false;

template <class F>
void launch(uint32_t nblocks, uint32_t nthreads, F&& body, bool thread0_last) {
    emu_gridDim = dim3(nblocks, 1, 1);
    emu_blockDim = dim3(nthreads, 1, 1);
    for (uint32_t b = 0; b < nblocks; ++b)
        for (uint32_t t = 0; t < nthreads; ++t) {
            if (thread0_last && b == 0 && t == 0) continue;
            emu_blockIdx = emu_idx(b);
            emu_threadIdx = emu_idx(t);
            body();
        }
    if (thread0_last) {
        emu_blockIdx = emu_idx(0);
        emu_threadIdx = emu_idx(0);
        body();
    }
}

// True when some pair on qubit t has both members present with a non-negligible bit-0 value:
// the situation in which the reference's Rx/Ry skip path corrupts its address book.
bool rxry_hazard(uint32_t t) {
    const uint32_t sh = table_d_.sh_[0];
    for (int32_t i = 0; i < table_d_.N_; ++i) {
        thash h = table_d_.ah_[sh + i];
        tkey k = table_d_.akvs_[sh + h].k;
        if (k < 0) continue;
        if ((k >> t) & 1) {
            const KV& p = table_d_.akvs_[sh + (k - (tkey(1) << t))];
            if (!ComplexManager::is_negligible(p.v)) return true;
        }
    }
    return false;
}

}  // namespace

extern "C" {

// Create the dense-capacity FC table for nq qubits (capacity 2^nq) and set |0...0>.
int refemu_create(uint32_t nq) {
    if (nq > 22) return -1;
    const uint32_t cap = 1u << nq;
    g_kv.assign(2 * size_t(cap), KV());
    g_ah.assign(2 * size_t(cap), -1);
    std::memset(&table_d_, 0, sizeof(table_d_));
    table_d_.akvs_ = g_kv.data();
    table_d_.a_exch_ = nullptr;
    table_d_.ah_ = g_ah.data();
    table_d_.N_st_ = 1;
    table_d_.capacity_st_ = cap;
    table_d_.Nb_ = cap;
    table_d_.bucket_size_ = 1;
    table_d_.capacity_ = cap;
    table_d_.flag_gpus_ = false;
    g_blocks = std::min<uint32_t>((cap - 1) / kThreads + 1, kMaxBlocks);
    launch(g_blocks, kThreads, [] { device_init_arrays(); }, false);
    launch(1, 1, [] { FC__::set_to_zero_quantum_state(); }, false);
    g_counter = 0;
    g_live = true;
    return 0;
}

void refemu_destroy(void) {
    g_kv.clear(); g_kv.shrink_to_fit();
    g_ah.clear(); g_ah.shrink_to_fit();
    g_live = false;
}

// kind: 0 X, 1 Y, 2 Z, 3 H, 4 Phase, 5 Rz, 6 Rx, 7 Ry (the engine's gate numbering).
// Returns 0, 1 when an Rx/Ry gate ran into the reference's address-book race, <0 on error.
int refemu_gate(int kind, uint32_t t, double par) {
    if (!g_live || t > 30) return -1;
    int hazard = 0;
    switch (kind) {
    case 0: launch(g_blocks, kThreads, [t] { FC__::gate_sq<0>(t); }, false); break;
    case 1: launch(g_blocks, kThreads, [t] { FC__::gate_sq<1>(t); }, false); break;
    case 2: launch(g_blocks, kThreads, [t] { FC__::gate_sq<2>(t); }, false); break;
    case 3: launch(g_blocks, kThreads, [t] { FC__::gate_sq<10>(t); }, false); break;
    case 4: launch(g_blocks, kThreads, [t, par] { FC__::gate_sq_par<0>(t, par); }, false); break;
    case 5: { double p = par / 2.; launch(g_blocks, kThreads, [t, p] { FC__::gate_sq_par<1>(t, p); }, false); break; }
    case 6: { hazard = rxry_hazard(t); double p = par / 2.;
              launch(g_blocks, kThreads, [t, p] { FC__::gate_sq_par<10>(t, p); }, false); break; }
    case 7: { hazard = rxry_hazard(t); double p = par / 2.;
              launch(g_blocks, kThreads, [t, p] { FC__::gate_sq_par<11>(t, p); }, false); break; }
    default: return -2;
    }
    launch(g_blocks, kThreads, [] { device_zero_arrays(); }, true);
    ++g_counter;
    return hazard;
}

// Number of address-book entries (the reference's N_), for diagnostics.
int64_t refemu_address_book_size(void) { return g_live ? int64_t(table_d_.N_) : -1; }

// Key-sorted readout of the non-negligible entries of the current half (table.cuh:47-75).
// Returns the count, -1 when cap is too small, -2 on a duplicate key.
int64_t refemu_get_state(uint64_t* keys, double* re, double* im, uint64_t cap) {
    if (!g_live) return -3;
    const uint32_t C = table_d_.capacity_;
    const uint32_t sh = (g_counter % 2 == 0) ? 0 : C;
    std::vector<std::pair<uint64_t, tvalue>> out;
    for (uint32_t i = 0; i < C; ++i) {
        const KV& kv = g_kv[sh + i];
        if (ComplexManager::is_negligible(kv.v)) continue;
        out.emplace_back(uint64_t(kv.k), kv.v);
    }
    std::sort(out.begin(), out.end(), [](auto& a, auto& b) { return a.first < b.first; });
    for (size_t i = 1; i < out.size(); ++i)
        if (out[i].first == out[i - 1].first) return -2;
    if (out.size() > cap) return -1;
    for (size_t i = 0; i < out.size(); ++i) {
        keys[i] = out[i].first; re[i] = out[i].second.r; im[i] = out[i].second.i;
    }
    return int64_t(out.size());
}

}  // extern "C"
