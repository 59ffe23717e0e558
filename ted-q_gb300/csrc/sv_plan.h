// sv_plan.h -- the compiled state-vector schedule shared by the host
// scheduler (sv_program.cpp) and the CUDA kernels (sv_kernels.cu).
//
// A circuit is executed as a sequence of *passes*.  A pass streams the whole
// state once through HBM in tiles of 2^m amplitudes: the tile of a pass is
// the set of amplitudes that differ only in the pass's m "tile bits" (the
// lowest ``c`` bits of the flat index are always tile bits so every tile is
// made of 2^c-amplitude contiguous runs).  Inside a tile, the gates of the
// pass run in *phases*: in a phase every thread holds 2^R amplitudes in
// registers -- the amplitudes that differ in the phase's R register bits --
// and applies all gates of the phase to them without touching shared memory.
// Between phases the tile is re-read from shared memory with another choice
// of register bits.
//
// Everything a kernel needs about one pass travels in one PassParams struct
// passed by value (``__grid_constant__``); the program needs no device memory.
#pragma once
#if defined(__CUDACC_RTC__)
typedef unsigned char uint8_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
#else
#include <stdint.h>
#include <stdlib.h>
#endif

namespace tedq {

constexpr int kMaxPhases = 24;
constexpr int kMaxPassGates = 160;
constexpr int kMaxMats = 128;
constexpr int kMaxFactors = 192;
constexpr int kMaxFixed = 96;
constexpr int kMaxTileBits = 16;
constexpr int kMaxStateBits = 34;
constexpr int kMaxRegUnits = 32;
constexpr int kMaxTidBits = 16;

// Register-phase gate kinds.
enum GateKind : uint8_t {
  GK_U1 = 0,    // dense 2x2 on register bit k0 (matrix: 4 entries)
  GK_D1 = 1,    // diagonal 2x2 on k0 (matrix: 2 entries)
  GK_X = 2,     // controlled bit flip of k0 (no matrix)
  GK_SWAP = 3,  // swap of register bits k0, k1 (no matrix)
  GK_RXT = 4,   // [[c, -i s], [-i s, c]]: c = M[0].re, s = -M[1].im (4 FMA/amplitude)
  GK_RYT = 5,   // [[c, -s], [s, c]]:      c = M[0].re, s = -M[1].re
  GK_PH = 6,    // diag(1, d): only the |1> half is multiplied (d = matrix entry 1)
  GK_H = 7,     // Hadamard (x0 + x1, x0 - x1) / sqrt(2) (no matrix)
  // Normalised rotations (global phase and scale dropped; uncontrolled only):
  // the gate divided by the larger of |c|, |s| costs one FMA per real
  // component.  Matrix entries: [0] = (coefficient, form), [1] = (scale, 0),
  // [2] = (running scale product of the pass up to this gate, 0).
  //   RXN form 0: [[1, -i t], [-i t, 1]]   form 1: [[i u, 1], [1, i u]]
  //   RYN form 0: [[1, -t], [t, 1]]        form 1: [[u, -1], [1, u]]
  // The pass multiplies its states by the total scale after the last one.
  GK_RXN = 8,
  GK_RYN = 9,
};

constexpr uint8_t kNoNorm = 0xFF;

// Generator kinds of the adjoint gradient: the gradient of a gate
// U(theta) with dU/dtheta = K U is 2 Re <lambda| K |psi> evaluated on the
// states after the gate.  K = -i/2 sigma (rotations) or i P1 (phases);
// the kernel returns coef * Im <lambda| G |psi> restricted to the control
// subspace with G = X, Y, Z or P1 = |1><1|.
enum GradKind : uint8_t { GR_NONE = 0, GR_X = 1, GR_Y = 2, GR_Z = 3, GR_P1 = 4 };

struct RGate {
  uint8_t kind;    // GateKind
  uint8_t k0, k1;  // register bit indices
  uint8_t cmask;   // controls (register-bit mask); all must be 1
  uint8_t mat;     // index into PassParams::mat
  uint8_t grad;    // GradKind (adjoint only)
  uint8_t pad[2];
  int32_t slot;    // parameter slot receiving the gradient, -1 = none
  float coef;      // gradient coefficient
};

// Factor ops: one factor produces a 2x2 matrix (dense or diagonal).
enum FactorOp : uint8_t {
  F_FIXED2 = 0,  // fixed dense 2x2 at fixed[fix .. fix+3]
  F_FIXD = 1,    // fixed diagonal at fixed[fix .. fix+1]
  F_RX = 2, F_RY = 3, F_RZ = 4, F_PHASE = 5, F_ROT = 6,
};

struct Factor {
  uint8_t op;
  uint8_t pad;
  int16_t fix;
  int32_t slot[3];  // parameter slots, -1 = use val
  double val[3];
};

// A matrix of a pass: the product F_last ... F_first of its factors.
struct MatDesc {
  uint8_t diag;    // 0: dense 2x2; 1: diagonal (2 entries); 2: diagonal with its
                   // global phase dropped, (1, d1 / d0); 3 / 4: normalised RX- /
                   // RY-type rotation (GK_RXN / GK_RYN entries)
  uint8_t nf;      // number of factors
  uint8_t f0;      // first factor index
  uint8_t dagger;  // 1: use the conjugate transpose (adjoint sweep)
};

struct CD { double re, im; };

enum PhaseType : uint8_t { PH_REG = 0, PH_DENSE = 1 };

struct Phase {
  uint8_t type;       // PhaseType
  uint8_t ntid;       // tid bits used for this phase's tile positions
  uint16_t g0, g1;    // RGate range [g0, g1) (PH_REG)
  // PH_REG: shared-memory unit offset (swizzled) of register unit j and of
  // thread-index bit b; unit address = XOR of the tid offsets ^ reg_off[j].
  uint16_t reg_off[kMaxRegUnits];
  uint16_t tid_off[kMaxTidBits];
  // PH_DENSE: one fixed k-qubit matrix applied directly in shared memory.
  uint8_t dk;          // 1..3
  uint8_t dpos[3];     // tile positions, dpos[0] = most significant matrix bit
  uint16_t dcmask;     // control mask over tile positions
  uint8_t dagger;
  // PH_REG: 1 = every warp touches the same shared-memory units as in the
  // previous register phase (same warp-index bits, the lane and register bits
  // permuted among themselves), so the transition needs only __syncwarp
  uint8_t wlocal;
  uint16_t dfix;       // first entry in fixed[] (4^dk entries, row-major)
  uint16_t pad2;
};

struct PassParams {
  uint8_t m;        // tile bits
  uint8_t c;        // low contiguous tile bits (chunk = 2^c amplitudes)
  uint8_t e;        // amplitudes per 16-byte unit = 2^e (1 for c64, 0 for c128)
  uint8_t R;        // register bits
  uint8_t n;        // state bits
  uint8_t n_outer;  // n - m
  uint8_t n_phases;
  uint8_t init;     // first pass of a forward sweep: 0 = read psi,
                    // 1 = generate |0..0>, 2 = read the shared initial state
  uint16_t n_gates, n_mats, n_factors, n_grad;
  uint8_t pad_bits;  // init == 2: low idle qubits added by padding
  uint8_t pipe;      // set per launch: 1 = persistent CTAs with a prefetched tile
                     // slot per thread group (G + 1 slots), 0 = one tile per CTA
  // normalised rotations: matrix of the last one (kNoNorm = none) and the
  // register phase whose end multiplies the states by the pass's scale
  uint8_t norm_last;
  uint8_t norm_phase;
  uint8_t hi[kMaxTileBits];      // global bit of tile bit c+i
  // Forward sweeps from |0...0>: qubits that no earlier pass has touched are
  // still |0>, so a tile whose base has any of these (outer) bits set is all
  // zero before and after the pass and is skipped (not read, computed or
  // written; the caller clears the state before the first pass).  0 for the
  // adjoint sweep and for a user-given initial state.
  uint64_t zero_outer;
  uint8_t outer[kMaxStateBits];  // global bit of outer-index bit i
  // Tile staging: thread tid stages units u = tid + k * 2^(m-R), k < 2^(R-e).
  // Global amplitude offset = tile base | OR of gtid[b] over set bits b of
  // tid | gk[k]; shared-memory unit = XOR of stid[b] ^ sk[k] (swizzled).
  uint64_t gtid[kMaxTidBits];
  uint64_t gk[kMaxRegUnits];
  uint32_t stid[kMaxTidBits];
  uint32_t sk[kMaxRegUnits];
  Phase phase[kMaxPhases];
  RGate gate[kMaxPassGates];
  MatDesc mat[kMaxMats];
  Factor factor[kMaxFactors];
  CD fixed[kMaxFixed];
};

#if defined(__CUDACC__)
#define TEDQ_HD __host__ __device__
#else
#define TEDQ_HD
#endif

// Shared memory of a pass kernel.  A CTA runs G thread groups of 2^(m-R)
// threads; each group works on one tile at a time.  Pipelined (P.pipe = 1):
// the CTA holds G + 1 tile slots, so that while the groups compute, the next
// tile is already arriving in the spare slot by asynchronous copies; one tile
// per CTA (P.pipe = 0): G = 1 and one slot.  After the slots: per group the
// pass matrices and (adjoint) the gradient sums, then one mbarrier per slot.
struct PipeLayout {
  uint32_t slot_bytes, mats_off, gacc_off, mbar_off, total;
};

TEDQ_HD inline int pipe_slots(const PassParams& P, int G) { return P.pipe ? G + 1 : 1; }

constexpr uint32_t kPipeSmemMax = 227u * 1024u;

TEDQ_HD inline PipeLayout pipe_layout(const PassParams& P, int G, bool adjoint) {
  PipeLayout L;
  const uint32_t amp = P.e == 1 ? 8u : 16u;  // bytes per amplitude (complex64 / complex128)
  const uint32_t T = 1u << (P.m - P.R);
  const uint32_t W = T >= 32u ? T / 32u : 1u;
  L.slot_bytes = (adjoint ? 2u : 1u) * (amp << P.m);
  uint32_t off = L.slot_bytes * (uint32_t)pipe_slots(P, G);
  L.mats_off = off;
  off += (uint32_t)G * (uint32_t)(P.n_mats > 0 ? P.n_mats : 1) * 4u * amp;
  off = (off + 15u) & ~15u;
  L.gacc_off = off;
  // FP64 sums [G][gates], then per-warp partials [G][W][gates] in the state's precision
  if (adjoint) off += (uint32_t)G * (uint32_t)(P.n_gates > 0 ? P.n_gates : 1) * (8u + W * (amp / 2u));
  off = (off + 15u) & ~15u;
  L.mbar_off = off;
  off += 8u * (uint32_t)pipe_slots(P, G);
  L.total = off;
  return L;
}

#if !defined(__CUDACC_RTC__)
// Launch variant of a specialised pass kernel: the tile pipeline (FwdPass /
// BwdPass) when every circuit has several tiles and the pass is short (at
// most 64 register gates) or arithmetic-heavy (at least 40 % dense or
// rotation gates, the kinds with two or more packed FMAs per amplitude);
// otherwise one tile per CTA (FwdTile / BwdTile).  Measured: the 20-qubit
// VQC (23-160 gates per pass, half of them rotations) runs faster pipelined
// in every pass; the 24-qubit MBL chain (60-160 Hadamard, CNOT and phase
// gates per pass, long code for little arithmetic) and small circuits whose
// tile is the whole state run faster one tile per CTA.  TEDQ_GB300_PIPE=0 / 1
// forces a variant (a measurement knob).  A pass whose two groups and three
// slots do not fit in shared memory (long complex128 adjoint passes) runs
// one tile per CTA: one pipelined group per SM would halve the warps.
inline bool pass_pipelined(const PassParams& P, bool adjoint) {
  const char* env = getenv("TEDQ_GB300_PIPE");
  if (env && (env[0] == '0' || env[0] == '1') && !env[1]) return env[0] == '1';
  if (P.n <= P.m) return false;
  PassParams Q = P;
  Q.pipe = 1;
  if ((2u << (P.m - P.R)) > 1024u || pipe_layout(Q, 2, adjoint).total > kPipeSmemMax) return false;
  if (P.n_gates <= 64) return true;
  int heavy = 0;
  for (int i = 0; i < P.n_gates; ++i) {
    const uint8_t k = P.gate[i].kind;
    heavy += (k == GK_U1 || k == GK_RXT || k == GK_RYT || k == GK_RXN || k == GK_RYN) ? 1 : 0;
  }
  return 5 * heavy >= 2 * P.n_gates;
}

// Shared memory of the one-tile-per-CTA variant: dynamic (the tile) and
// static (matrices, per-warp gradient slots).
inline uint32_t tile_dynamic_smem(const PassParams& P, bool adjoint) {
  return (adjoint ? 32u : 16u) << (P.m - P.e);
}
inline uint32_t tile_static_smem(const PassParams& P, bool adjoint) {
  const uint32_t amp = P.e == 1 ? 8u : 16u;
  return (uint32_t)kMaxMats * 4u * amp + (adjoint ? 8u * (uint32_t)kMaxPassGates * (amp / 2u) : 0u);
}

// Pipelined launches: two groups (three slots) when they fit in shared
// memory, else one group with a double-buffered tile; TEDQ_GB300_PIPE_GROUPS=1
// asks for one group (a measurement knob).  One tile per CTA: one group.
inline int pipe_groups(const PassParams& P, bool adjoint) {
  if (!P.pipe) return 1;
  const uint32_t T = 1u << (P.m - P.R);
  const char* env = getenv("TEDQ_GB300_PIPE_GROUPS");
  const int want = (env && env[0] == '1') ? 1 : 2;
  if (want == 2 && 2u * T <= 1024u && pipe_layout(P, 2, adjoint).total <= kPipeSmemMax) return 2;
  return 1;
}
#endif

// Unit-level shared-memory swizzle: the 16-byte unit u of a tile is stored at
// u ^ fold3(u >> 3) where fold3 xors the 3-bit groups.  The map is linear over
// GF(2), so offsets of disjoint bit sets combine with XOR.
TEDQ_HD inline uint32_t swz_unit(uint32_t u) {
  uint32_t v = u >> 3, f = 0;
  while (v) { f ^= v & 7u; v >>= 3; }
  return u ^ f;
}

}  // namespace tedq
