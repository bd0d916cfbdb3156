// Device-side tables and helpers shared by the SUS2 GPU kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sus2g {

constexpr int kWarp = 32;
constexpr int kMaxK = 8;        // radial channels a warp-per-atom pass keeps in registers
constexpr int kMaxB = 16;       // Chebyshev basis size kept in registers

// Device error codes recorded by kernels (first error wins); the host turns them into messages.
enum DeviceError : int {
  kErrNone = 0,
  kErrEdgeCapacity = 1,   // a neighbour list exceeded the capacity the builder planned for
  kErrImageRange = 2,     // periodic image index outside the packed range
  kErrReverseEdge = 3,    // a directed edge had no reverse partner
  kErrBadDistance = 4,    // zero or non-finite edge length
  kErrBadPosition = 5,    // a non-finite atom coordinate in a periodic frame
  kErrBadSpecies = 6,     // an atom species index outside [0, C)
  kErrAsyncCopy = 7,      // a bulk asynchronous copy into shared memory did not complete in time
};

__device__ __forceinline__ void record_error(int* flag, int code) {
  if (flag) atomicCAS(flag, 0, code);
}

// Edge geometry record (dx, dy, dz, r) in the compute precision.
struct __align__(16) EdgeF { float x, y, z, w; };
struct __align__(32) EdgeD { double x, y, z, w; };
template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = EdgeF; };
template <> struct Vec4<double> { using type = EdgeD; };

// Per-atom graph program of one pass: the rank contraction and the product graph, forward and
// reverse, as steps of lane-balanced work.  A step adds to one node array (v forward, adj reverse)
//     T[target] += sum over a term list of c * X[a] * v[b]     (X = v forward, adj reverse)
// where node M is a constant 1 (so a contraction row w v[src] is the term (src, M, w)).  Each
// step's term lists are cut into chunks of about (terms / 32) terms, and the chunks are dealt to
// the lanes longest first onto the least-loaded lane (host side).  A lane's chunks form one term
// stream; the streams are stored lane-major -- row i holds term i of every lane, 32 consecutive
// records -- so that a warp reads each row with one coalesced access, and are padded to the
// step's longest stream with zero terms.  The last term of a chunk carries its flush target: the
// node the chunk sum is added to, or a partial slot when the list was cut into several chunks;
// the lanes combine the slots of such lists in slot order after the step (deterministic).
template <typename Real> struct ProgRec;
template <> struct __align__(16) ProgRec<float> { unsigned ab; int flush; float c, pad; };   // ab = a | b << 16
template <> struct __align__(16) ProgRec<double> { unsigned ab; int flush; double c; };
// flush: kProgNoFlush, a node index >= 0, or -(slot + 2) for a partial slot
constexpr int kProgNoFlush = -1;

// One program record through the read-only data path (the records are written by host uploads
// only): as a non-coherent load it may be issued ahead of the node stores of earlier records,
// which a plain load through the generic pointer may not pass.
template <typename Real>
__device__ __forceinline__ ProgRec<Real> load_rec(const ProgRec<Real>* p) {
  const int4 w = __ldg(reinterpret_cast<const int4*>(p));
  ProgRec<Real> r;
  r.ab = static_cast<unsigned>(w.x);
  r.flush = w.y;
  if constexpr (sizeof(Real) == 4) {
    r.c = __int_as_float(w.z);
    r.pad = __int_as_float(w.w);
  } else {
    r.c = __hiloint2double(w.w, w.z);
  }
  return r;
}

template <typename Real>
struct GraphProg {
  int nsteps = 0, nfwd = 0;      // forward steps [0, nfwd), reverse steps [nfwd, nsteps)
  int max_parts = 0;             // partial slots any step uses
  const int4* steps = nullptr;   // {first row, rows, comb begin, (comb end << 1) | reverse}
  const int4* comb = nullptr;    // {node, slot begin, slot end, 0}
  const ProgRec<Real>* rows = nullptr;  // [row][32]
};

// Per-pass tables: the outer (energy) pass and the Effect gate pass share this layout.
template <typename Real>
struct PassTables {
  const Real* coeff;      // F x B Chebyshev coefficients of R_mu
  const Real* scal;       // warp: slope at [2 sb C^2 + pair], shift at [(2 sb + 1) C^2 + pair]
  const Real* wcenter;    // C x F centre factor  (tau or gate type)
  const Real* wsource;    // C x F source factor  (tau or gate type)
  const Real* wadd;       // C x F Effect additive factor alpha (outer pass of gated models), else null
  // ranked K contraction, forward grouped by destination node
  int ndst;
  const int* dst_node;    // [ndst]
  const int* dst_begin;   // [ndst + 1]
  const int* dst_src;     // basic index
  const Real* dst_w;
  // reverse grouped by basic index
  const int* src_begin;   // [NB + 1]
  const int* src_dst;
  const Real* src_w;
  // per-atom product graph schedule (see model.cpp build_schedule)
  int levels;
  const int* level_begin;   // [levels + 1]
  const int* out_nodes;
  const int* out_begin;
  const int* fprod_a;
  const int* fprod_b;
  const Real* fprod_c;
  const int* rlevel_begin;  // [levels + 1] (levels >= 1; level 0 holds sources)
  const int* in_nodes;
  const int* in_begin;
  const int* rprod_out;
  const int* rprod_other;
  const Real* rprod_c;
  GraphProg<Real> prog;   // the same contraction and graph as a lane-balanced program (E/F/virial passes)
};

// Parameter-vector offsets (the trainer's Coeff() order) and the gradient-only tables of one pass.
struct PassGradLayout {
  int coeff_off, coeff_stride;   // offset of R_mu's Chebyshev row mu: coeff_off + mu * coeff_stride
  int scal_off;                  // offset of this pass's warp block
  int wc_off, wc_mu_stride, wc_t_stride;  // factor (t, mu) at wc_off + t * wc_t_stride + mu * wc_mu_stride
  int add_off;                   // Effect alpha block (t * F + mu), -1 if none
  int rw_off;                    // rank weight block, -1 if none (weights fixed at 1)
  int nw;                        // number of rank weights
  const int* w_begin;            // [nw + 1] rows of each rank weight
  const int* w_src;              // basic index of the row
  const int* w_dst;              // contraction node of the row
};

struct GradLayout {
  PassGradLayout outer, gate;
  int shift_off, species_off, linear_off, gate_w_off, nparams;
};

template <typename Real>
struct DevModel {
  int C, L, K, B, F, H, M, NB, S, Q, nblk, scaling_mode;
  Real rmax, rang, scaling;
  int split, poly, cutoff_p, gated, species_readout;
  const int* basic_of;      // K x H canonical (k, l*l+l+m) -> basic index, -1 when absent
  PassTables<Real> outer, gate;
  const Real* linear;       // readout weights (S or C x S)
  const double* species;    // C
  const double* shift;      // C
  const int* scalar_map;    // S
  const Real* gate_wmat;    // F x Q gate projection h = W g
  const int* gate_nodes;    // Q
  GradLayout grad;          // parameter-gradient layout
  int prog_parts;           // partial slots of the larger of the two passes' graph programs
};

__device__ __forceinline__ int warp_lane() { return threadIdx.x & (kWarp - 1); }

// Programmatic dependent launch (griddepcontrol, sm_90 and later).  A kernel launched with the
// programmatic-serialization attribute may start while the previous kernel of its stream is still
// draining, once every block of that kernel has called pdl_launch_dependents() or exited; it must
// call pdl_wait() -- which returns when all its prerequisite grids have completed and their memory
// is visible -- before it reads anything those grids (or earlier work) wrote, and every block must
// execute it so that the grid's completion implies its prerequisites' completion.  Without the
// attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// 1-D bulk asynchronous copies (the TMA unit's non-tensor mode) from this GPU's global memory
// into the CTA's shared memory, completed on an mbarrier with a transaction count.  Addresses on
// both sides 16-byte aligned, sizes multiples of 16 bytes.  Nothing here uses a cluster peer: the
// shared::cluster destination is the issuing CTA's own shared memory.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
// one arrival per phase; visible to the async proxy after the fences
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned arrivals) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(arrivals) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// this thread's arrival for the phase, announcing `bytes` of copies that complete it
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// orders this thread's earlier generic shared-memory accesses (and, after a warp barrier, those of
// the threads it synchronised with) before its later async-proxy operations
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// global -> shared bulk copy, completing `bytes` of the barrier's transaction count
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the phase of the given parity to complete, for at most about 2^31 clocks (~1 s);
// false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  const long long t0 = clock64();
  for (int it = 0; it < (1 << 26); ++it) {
    if (mbar_test(bar, parity)) return true;
    if (clock64() - t0 > (1ll << 31)) break;
  }
  return false;
}

// kernel<<<grid, block, smem, stream>>>(args...), with the programmatic-serialization attribute
// when pdl is set.  Returns the launch status.
template <typename... P, typename... A>
inline cudaError_t launch_kernel(bool pdl, void (*kernel)(P...), dim3 grid, dim3 block, size_t smem,
                                 cudaStream_t stream, A&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = pdl ? attr : nullptr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

// kernel<<<grid, block, smem, stream>>>(args...) at the given scheduling priority (a stream
// priority value; lower is more urgent): its blocks are placed ahead of lower-priority pending
// blocks when SM resources free up, also inside a captured graph.
template <typename... P, typename... A>
inline cudaError_t launch_kernel_priority(int priority, void (*kernel)(P...), dim3 grid, dim3 block, size_t smem,
                                          cudaStream_t stream, A&&... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributePriority;
  attr[0].val.priority = priority;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Compensated FP32 accumulation (Knuth two-sum; the running error is kept in lo): sums of FP32
// terms with close to FP64 accuracy without FP64 arithmetic, which runs at 1/64 of the FP32 rate
// on this GPU.  Every step is an explicitly rounded operation (__fadd_rn / __fsub_rn / __fmul_rn),
// which the compiler never fuses with a neighbouring multiply: the sums are the same bits in every
// kernel instantiation (register budget) that inlines them.
__device__ __forceinline__ void csum_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x);
  const float bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb)));
  hi = s;
}
// x * y added exactly (product split by an FMA: p + e == x * y).
__device__ __forceinline__ void csum_add_prod(float& hi, float& lo, float x, float y) {
  const float p = __fmul_rn(x, y);
  const float e = fmaf(x, y, -p);
  csum_add(hi, lo, p);
  lo = __fadd_rn(lo, e);
}
// Warp total of compensated partials (fixed butterfly order), left as (hi, lo) on every lane.
__device__ __forceinline__ void warp_csum_pair(float& hi, float& lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
    csum_add(hi, lo, oh);
    lo = __fadd_rn(lo, ol);
  }
}
// The same total returned in FP64 on every lane.
__device__ __forceinline__ double warp_csum(float hi, float lo) {
  warp_csum_pair(hi, lo);
  return double(hi) + double(lo);
}

// p[0] + p[stride] + ... + p[(n - 1) stride], added in that order, with DEPTH loads in flight
// ahead of the adds (a column of a row-major per-edge array, summed over one centre's edges).
template <typename Real, int DEPTH = 8>
__device__ __forceinline__ Real column_sum(const Real* p, size_t stride, int n) {
  Real s = Real(0);
  int i = 0;
  for (; i + DEPTH <= n; i += DEPTH) {
    Real x[DEPTH];
#pragma unroll
    for (int q = 0; q < DEPTH; ++q) x[q] = p[static_cast<size_t>(i + q) * stride];
#pragma unroll
    for (int q = 0; q < DEPTH; ++q) s += x[q];
  }
  for (; i < n; ++i) s += p[static_cast<size_t>(i) * stride];
  return s;
}

// The F columns of a row-major per-edge array [n][F] (F <= 64) summed over the rows into dst[F]:
// lane c sums columns c and c + 32 side by side, each row after row in order (the sums of
// column_sum), sixteen loads in flight.
template <typename Real>
__device__ __forceinline__ void column_sums_2(const Real* p, int F, int n, Real* dst, int lane) {
  const int mu0 = lane, mu1 = lane + 32;
  const bool on0 = mu0 < F, on1 = mu1 < F;
  Real s0 = Real(0), s1 = Real(0);
  int i = 0;
  for (; i + 8 <= n; i += 8) {
    Real x0[8], x1[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      x0[q] = on0 ? p[static_cast<size_t>(i + q) * F + mu0] : Real(0);
      x1[q] = on1 ? p[static_cast<size_t>(i + q) * F + mu1] : Real(0);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) { s0 += x0[q]; s1 += x1[q]; }
  }
  for (; i < n; ++i) {
    if (on0) s0 += p[static_cast<size_t>(i) * F + mu0];
    if (on1) s1 += p[static_cast<size_t>(i) * F + mu1];
  }
  if (on0) dst[mu0] = s0;
  if (on1) dst[mu1] = s1;
}

// Warp index of the scaling block for radial function (k, l) (sus2_sl_kernel.cpp:198).
__device__ __forceinline__ int scaling_block(int mode, int k, int l, int Lp) {
  return mode == 2 ? k : (mode == 1 ? l : (mode == 0 ? 0 : k * Lp + l));
}

}  // namespace sus2g
