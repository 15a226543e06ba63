// Internal structures shared by the host library (gpb_host.cpp) and the CUDA
// kernels (gpb_kernels.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gpb {

// Instances are stored in packs of LANES (one warp, one instance per lane).
// Every per-instance array is "lane-interleaved": element e of the instance in
// lane l of a pack lives at base_row(pack) * LANES + e * LANES + l, so that the
// 32 lanes of a warp touch 32 consecutive words.
constexpr int LANES = 32;

// Topology word 0 of a body: joint type | parent << 4 | qo << 12 | vo << 22.
// Word 1: flags (bits 0-7) | first contact << 8 | contact count << 16.
enum BodyFlags : uint32_t {
  BF_INIT_ROT_IDENTITY = 1u << 0,  // init rotation is the identity
  BF_AXIS_PRINCIPAL = 1u << 1,     // axis is ±x, ±y or ±z (index in bits 2-3, sign bit 4)
  BF_AXIS_NEG = 1u << 4,
  BF_BRANCH = 1u << 5,             // some child is not the next body: keep X, V, A in scratch
  BF_SPRING = 1u << 6,             // prismatic spring
  BF_DIAG_INERTIA = 1u << 7,       // body-frame moment is diagonal
};
__host__ __device__ inline uint32_t bf_axis_index(uint32_t flags) { return (flags >> 2) & 3u; }

// Doubles (and floats) of one body in the topology table.
// Rinit (9, row-major), tinit (3), axis (3), inertia (10), spring (2), armature,
// cuboid collider sizes (3)
constexpr int TOPO_D = 31;
constexpr int TD_RINIT = 0, TD_TINIT = 9, TD_AXIS = 12, TD_INERTIA = 15, TD_SPRING = 25, TD_ARMATURE = 27,
              TD_CUBOID = 28;
// Second topology word: flags (bits 0-7), first contact (8-15), contact count
// (16-23), cuboid slot + 1 (24-27; 0 = no collider).
constexpr int W1_CUBOID_SHIFT = 24;
// Per-slot cuboid record in scratch (FP64 rows): world rotation (9), centre (3),
// world twist about the world origin (ω 3, v 3), sizes (3), accumulated world
// wrench about the world origin (moment 3, force 3).
constexpr int UREC_D = 27;
constexpr int UR_R = 0, UR_T = 9, UR_W = 12, UR_V = 15, UR_DIM = 18, UR_MOM = 21, UR_FRC = 24;
constexpr int CTC_D = 6;    // location (3), k, radius, damping
constexpr int HS_D = 8;     // point (3), normal (3), alpha, mu
constexpr int LANE_I = 8;   // per-lane ints: instance, nb, nq, nv, nc, nh, contact model, cuboids

struct PackDesc {
  int32_t count, nb, nq, nv, nc, nh, chain, minnv;  // minnv: smallest DOF count of its lanes
  int32_t nu;   // largest cuboid-collider count of its lanes
  int32_t mvs;  // velocity stepping: largest potential contact count of its lanes
                // (points × half-spaces + cuboid pairs), 0 = none
  int32_t kind;  // mechanism kind of every lane, for the instantiation of the
                 // articulated-body passes (0 general, 1 planar chain, 2 floating tree;
                 // see gpb_aba.cuh); general unless every pack of the batch has one kind
  // bases in rows (one row = LANES elements)
  int64_t topo;   // topology bodies (2 int words / TOPO_D reals per body)
  int64_t ctc;    // contacts
  int64_t hs;     // half-spaces
  int64_t q, v;   // state (doubles)
  int64_t lane;   // per-lane ints
  int64_t scr;    // scratch, in rows of 8-byte words
  int64_t vs;     // velocity-stepping scratch, in rows of 8-byte words
};

// Scratch sub-array offsets (rows of 8-byte words; R-typed arrays use the same
// row pitch so that the float and double kernels share one layout).
struct ScratchLayout {
  int32_t X, V, A, S, I, F, C, AI, DU, RF, M, D, rhs, q0, v0, qs, vs, facc, tau, cf, U, VW, FD, total;
};
__host__ __device__ inline ScratchLayout scratch_layout(int nb, int nq, int nv, int nc, int nu) {
  ScratchLayout s;
  int o = 0;
  s.X = o; o += 12 * nb;
  s.V = o; o += 6 * nb;
  s.A = o; o += 6 * nb;
  s.S = o; o += 6 * nv;
  s.I = o; o += 12 * nb;  // world inertia (10) or, in link coordinates, (Rrel, t) (12)
  s.F = o; o += 6 * nb;
  s.C = o; o += 10 * nb;  // link coordinates: composite inertia accumulated from branches
  s.AI = o; o += 21 * nb; // articulated-body algorithm: articulated inertias (FP64 or double-float)
  s.DU = o; o += 11 * nv; // articulated-body algorithm: U, 1/D, u per DOF (FP64)
  s.RF = o; o += 12 * nb; // articulated-body algorithm: (Rrel, t) in the sweep precision
  const int nT = (nv + 3) / 4;  // mass matrix in 4x4 tiles, n padded to 4 nT
  s.M = o; o += nT * (nT + 1) / 2 * 16;
  s.D = o; o += 4 * nT;
  s.rhs = o; o += 4 * nT;
  s.q0 = o; o += nq;
  s.v0 = o; o += nv;
  s.qs = o; o += nq;
  s.vs = o; o += nv;
  s.facc = o; o += nv;
  s.tau = o; o += nv;
  s.cf = o; o += 3 * nc;
  s.U = o; o += nu > 1 ? UREC_D * nu : 0;  // cuboid records (pairs need two)
  // mixed articulated-body algorithm of contact mechanisms: FP64 body velocities of branch bodies
  s.VW = o; o += (nc > 0 || nu > 1) ? 6 * nb : 0;
  // mixed articulated-body algorithm of contact mechanisms: FP64 bias forces.  They
  // cannot share F with the FP32 bias forces of the pack's other lanes: an FP32
  // row fills the first half of the bytes of the FP64 row of the same index,
  // i.e. the FP64 elements of lanes 0-15.
  s.FD = o; o += (nc > 0 || nu > 1) ? 6 * nb : 0;
  s.total = o;
  return s;
}

// Velocity-stepping scratch of one pack (rows of 8-byte words, lane-interleaved),
// for up to mc contacts (m = 3 mc rows of the contact Jacobian) and nv DOF.
struct VSLayout {
  int32_t mc, m;
  int32_t ct;              // contacts: normal (3), point (3), body a, body b
  int32_t J, Y;            // J (m × nv, row-major) and Y = (M⁻¹ Jᵀ)ᵀ (m × nv)
  int32_t P, H;            // the scaled program's P and the Newton matrix (m × m)
  int32_t W, Wi, eta;      // per cone: NT scaling W, W⁻¹ (9 each), η
  int32_t qv, y, z, r, lam, dya, dza, dy, dz, rs, rhs, ds;  // m each
  int32_t vf, qdd;         // nv each: free velocity, its acceleration
  int32_t total;
};
__host__ __device__ inline VSLayout vs_layout(int nv, int mc) {
  VSLayout s;
  const int m = 3 * mc;
  int o = 0;
  s.mc = mc;
  s.m = m;
  s.ct = o; o += 8 * mc;
  s.J = o; o += m * nv;
  s.Y = o; o += m * nv;
  s.P = o; o += m * m;
  s.H = o; o += m * m;
  s.W = o; o += 9 * mc;
  s.Wi = o; o += 9 * mc;
  s.eta = o; o += mc;
  s.qv = o; o += m;
  s.y = o; o += m;
  s.z = o; o += m;
  s.r = o; o += m;
  s.lam = o; o += m;
  s.dya = o; o += m;
  s.dza = o; o += m;
  s.dy = o; o += m;
  s.dz = o; o += m;
  s.rs = o; o += m;
  s.rhs = o; o += m;
  s.ds = o; o += m;
  s.vf = o; o += nv;
  s.qdd = o; o += nv;
  s.total = o;
  return s;
}

// Serving: the job of one lane slot (pack * LANES + lane) of a server's pool.
// The step kernel runs min(K, steps_left) steps of the slot's request with the
// request's own step size, integrator and control law, then advances
// steps_left / step_index.
struct LaneJob {
  int64_t steps_left;  // steps still to run (0 = idle slot, or a job that failed)
  int64_t step_index;  // steps the request has run (its step counter for the open-loop draw)
  double dt, sigma, kp, kd;
  uint32_t seed;
  int32_t control;     // GPB_CONTROL_*
  int32_t resample;
  int32_t integrator;
  int32_t tau_mode;    // host control: 1 = tau_in holds the request's torques
  int32_t chunk;       // steps per launch of this slot (0 = the launch's K)
};
constexpr int LANE_JOB_WORDS = (int)(sizeof(LaneJob) / 8);
static_assert(sizeof(LaneJob) % 8 == 0, "LaneJob is written as 8-byte words");
static_assert(offsetof(LaneJob, step_index) == 8, "the server gathers step_index as word 1");

// Everything a kernel launch needs (device pointers).
struct DeviceBatch {
  int32_t npacks;
  const PackDesc* packs;
  const uint32_t* topoW;   // 2 words per body
  const double* topoD;
  const float* topoF;
  const int32_t* ctcI;     // body (0-based) | original index << 8
  const double* ctcD;
  const float* ctcF;
  const double* hsD;
  const float* hsF;
  const int32_t* laneI;
  int32_t* status;         // one int per lane slot (pack * LANES + lane)
  int64_t* done;           // steps completed in the last simulate launch, per slot
  double* q;
  double* v;
  double* tau_in;          // host torques or PD targets (pack layout)
  double* scratch;
  const int64_t* qmap;     // pack slot -> flat user index (-1 = padding)
  const int64_t* vmap;
  const int64_t* cmap;     // contact slot (3 per contact) -> flat user index
  int64_t nq_total, nv_total, nc_total;
  int32_t* queue;          // persistent-kernel work counters: [0] per-warp packs, [1] block packs
  int32_t algorithm;       // GPB_ALGO_CRBA or GPB_ALGO_ABA
  double gravity;          // m/s² along −z (9.81 unless set)
  int32_t plain;           // 1: no contact points, no prismatic springs (free_velocity)
  double* vscratch;        // velocity-stepping scratch (PackDesc::vs), null until first used
  // serving pool only (all null for a batch)
  LaneJob* jobs;           // per-slot jobs
  const int32_t* active;   // packs to run in this launch (nactive of them)
  int32_t nactive;
  int32_t* finished;       // slots whose job ended (done or failed) in this launch
  int32_t* nfinished;
};

// Scatter of 4- or 8-byte words into up to 16 device arrays: entry k writes
// bits[k] to element (key[k] & 0xffffffffffff) of target (key[k] >> 56).
struct ScatterTarget {
  void* base;
  int64_t count;  // elements
  int32_t bytes;  // 4 or 8
  int32_t pad;
};
struct ScatterTable {
  ScatterTarget t[16];
  int32_t n;
};

struct StepParams {
  double dt;
  int64_t K;
  int64_t step0;
  int32_t integrator;
  int32_t precision;
  int32_t control;
  uint32_t seed;
  int32_t resample;
  double sigma, kp, kd;
  int64_t record_every;
  double* history;      // device, [K/record_every][nq_total + nv_total]
  double* qdd_out;      // dynamics-only: user-order q̈ (device)
  double* cforce_out;   // dynamics-only: user-order contact forces (device)
  int32_t tau_mode;     // dynamics/step: 0 = zero torque, 1 = tau_in holds torques
  int32_t ncoop;        // packs [0, ncoop) are stepped by a whole 4-warp block
  int32_t free_velocity;  // dynamics-only: write v + vfree_dt·q̈ (no contacts, no springs)
  double vfree_dt;
  int32_t group;        // body-parallel mapping: lanes per instance (launch_simulate_group)
  int32_t group_nvp;    // body-parallel mapping: largest DOF count of the batch
};

// Launchers (gpb_kernels.cu).  All return a cudaError_t.
// warps_per_sm: resident warps per SM of the persistent grid (0 = the
// occupancy limit; otherwise rounded to whole 4-warp blocks and capped by it).
cudaError_t launch_simulate(const DeviceBatch& b, const StepParams& p,
                            int num_sms, int warps_per_sm, cudaStream_t s);
// Body-parallel mapping of serial chains (gpb_group.cuh): p.group lanes per
// instance (2 … 32 lanes of a warp, or 128: a 4-warp block), bodies_per_lane
// = 1 or 2 (p.group · bodies_per_lane ≥ every instance's body count), FP64.
cudaError_t launch_simulate_group(const DeviceBatch& b, const StepParams& p, int bodies_per_lane, int num_sms,
                                  cudaStream_t s);
cudaError_t launch_dynamics(const DeviceBatch& b, const StepParams& p, cudaStream_t s);
// Resident warps per SM the step kernel of `precision` can hold (registers).
cudaError_t simulate_max_warps_per_sm(int precision, int* warps);
cudaError_t launch_scatter(const int64_t* map, int64_t slots, const double* src, double* dst,
                           cudaStream_t s);
cudaError_t launch_gather(const int64_t* map, int64_t slots, const double* src, double* dst,
                          cudaStream_t s);
cudaError_t launch_scatter_words(const ScatterTable& table, const uint64_t* key, const uint64_t* bits,
                                 int64_t n, cudaStream_t s);
// dst[k] = src[idx[k]] for 4- or 8-byte elements.
cudaError_t launch_gather_words(const void* src, int bytes, const int64_t* idx, int64_t n, void* dst,
                                cudaStream_t s);
// gpb_collide_cuboids: n cuboid pairs (device arrays; pose 7 / sizes 3 doubles
// per cuboid), one thread per pair.
cudaError_t launch_collide(int64_t n, const double* pose_a, const double* size_a, const double* pose_b,
                           const double* size_b, int32_t* result, double* cp_a, double* cp_b, int num_sms,
                           cudaStream_t s);
// gpb_dynamics_static: the dynamics kernel with its scratch in the library's
// static device array (cudaErrorInvalidValue if scratch_words exceeds it).
cudaError_t launch_dynamics_static(const DeviceBatch& b, int device, int64_t scratch_words,
                                   int precision, const double* q, const double* v,
                                   const double* tau, double* qdd, cudaStream_t s);

// Open-loop torque draw shared bit for bit by host and device.
__host__ __device__ double open_loop_tau(uint32_t seed, int64_t inst, int64_t block, int32_t dof,
                                         double sigma);

}  // namespace gpb
