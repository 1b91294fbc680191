// sm_103a kernels of the box-QP engine.
//
// Hot path (one launch per FISTA iteration, graph-replayed):
//   step_kernel   fused CSR SpMV g = Q w, gradient step, clamp to [l,u], momentum update
//                 w+ = x+ + beta (x+ - x): reads w from one ping-pong buffer and writes the
//                 other, so no separate gradient array or second launch is needed
//                 (the reference uses csr_product + fista_step, src/cuda_box.cu:16-21,29).
//   check_kernel  FP64 verification of check_qp_solution (src/qp_admm.cpp:63-117) as block
//                 reductions: objective, primal residual, projected stationarity, dual bound,
//                 active-set signature; the last tile of each instance reduces that instance's
//                 tile partials in a fixed order (deterministic, independent of co-scheduled
//                 instances) and advances the instance's state machine.
//   polish_*/cg_* FP64 conjugate gradient on the free set Q_FF x_F = -c_F - Q_FA x_A (mixed).
//
// Memory-bound design: SpMV streams values/columns once per iteration with read-only loads;
// rows are processed by the SpMV structure the tuning table picks per instance (block- or
// warp-staged, or sub-warps of LANES lanes), one step kernel per (precision, structure);
// FP64 arithmetic is kept out of the FP32 iterations (GB300's FP64 rate is ~1/64 of FP32), and
// FP64 epilogues and reductions run on full warps (an FP64 warp instruction costs the same
// whatever its active lanes).
#include "kernels.cuh"
#include "fpbits.h"

#include <atomic>
#include <cmath>
#include <cstdio>
#include <type_traits>

namespace bqp {
namespace {

#define kInf (__longlong_as_double(0x7ff0000000000000LL))

__device__ __forceinline__ int64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return static_cast<int64_t>(t);
}

// std::max / std::min semantics of the reference.
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smaxf(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float sminf(float a, float b) { return (b < a) ? b : a; }

template <class T>
__device__ __forceinline__ T shfl_xor(T v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
template <class T>
__device__ __forceinline__ T shfl_idx(T v, int src) { return __shfl_sync(0xffffffffu, v, src); }
template <>
__device__ __forceinline__ float2 shfl_xor<float2>(float2 v, int o) {
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}
template <>
__device__ __forceinline__ float2 shfl_idx<float2>(float2 v, int src) {
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

template <int LANES, class T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) v += shfl_xor(v, o);
    return v;
}

// ---- check / CG accumulators ---------------------------------------------------------------------
// Sums in plain FP64, maxima of non-negative doubles as unsigned bit patterns.
__device__ __forceinline__ unsigned long long dbits(double v) {
    return static_cast<unsigned long long>(bits64(v));
}
__device__ __forceinline__ double bdouble(unsigned long long b) { return __longlong_as_double(static_cast<long long>(b)); }
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) { return a < b ? b : a; }

struct Acc {
    double obj, bnd, sep, a;
    unsigned long long stat, prim, b;
    unsigned hash;
    int nact;
    int flags;
};
__device__ __forceinline__ Acc acc_identity() {
    Acc a;
    a.obj = 0; a.bnd = 0; a.sep = 0; a.a = 0;
    a.stat = 0; a.prim = 0; a.b = 0; a.hash = 0;
    a.nact = 0; a.flags = 0;
    return a;
}
__device__ __forceinline__ Acc combine(const Acc& x, const Acc& y) {
    Acc r;
    r.obj = x.obj + y.obj;
    r.bnd = x.bnd + y.bnd;
    r.sep = x.sep + y.sep;
    r.a = x.a + y.a;
    r.stat = umax64(x.stat, y.stat);
    r.prim = umax64(x.prim, y.prim);
    r.b = umax64(x.b, y.b);
    r.hash = x.hash ^ y.hash;
    r.nact = x.nact + y.nact;
    r.flags = x.flags | y.flags;
    return r;
}
__device__ __forceinline__ Acc shfl_acc(const Acc& x, int o) {
    Acc r;
    r.obj = shfl_xor(x.obj, o); r.bnd = shfl_xor(x.bnd, o); r.sep = shfl_xor(x.sep, o); r.a = shfl_xor(x.a, o);
    r.stat = shfl_xor(x.stat, o); r.prim = shfl_xor(x.prim, o); r.b = shfl_xor(x.b, o);
    r.hash = shfl_xor(x.hash, o);
    r.nact = shfl_xor(x.nact, o);
    r.flags = shfl_xor(x.flags, o);
    return r;
}

// Fixed-order block reduction; the result is valid in thread 0.
__device__ Acc block_reduce(Acc v) {
    __shared__ Acc warp_part[kBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = combine(v, shfl_acc(v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_part[warp] = v;
    __syncthreads();
    if (warp == 0) {
        Acc w = lane < kBlock / 32 ? warp_part[lane] : acc_identity();
#pragma unroll
        for (int o = (kBlock / 64); o > 0; o >>= 1) w = combine(w, shfl_acc(w, o));
        v = w;
    }
    __syncthreads();
    return v;
}

// The check's reduction: the two FP64 sums it always needs (objective, tangent bound), the
// separable bound only for the diagonal dual-gap gate (GATE, a template parameter so that no
// FP64 addition runs for it otherwise), and the integer fields; the CG fields (a, b) stay out.
template <bool GATE>
__device__ __forceinline__ Acc combine_check(const Acc& x, const Acc& y) {
    Acc r = x;
    r.obj = x.obj + y.obj;
    r.bnd = x.bnd + y.bnd;
    if (GATE) r.sep = x.sep + y.sep;
    r.stat = umax64(x.stat, y.stat);
    r.prim = umax64(x.prim, y.prim);
    r.hash = x.hash ^ y.hash;
    r.nact = x.nact + y.nact;
    r.flags = x.flags | y.flags;
    return r;
}
// The integer fields over the warp (xor tree, integer pipes).
__device__ __forceinline__ void warp_ints(Acc& v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.stat = umax64(v.stat, shfl_xor(v.stat, o));
        v.prim = umax64(v.prim, shfl_xor(v.prim, o));
        v.hash ^= shfl_xor(v.hash, o);
        v.nact += shfl_xor(v.nact, o);
        v.flags |= shfl_xor(v.flags, o);
    }
}
// Block reduction of the check fields in a fixed order; valid in thread 0.  The FP64 sums go
// through shared memory: one warp adds each lane's 8 values (thread t: lane t % 32, in order of
// t), then an xor tree over the warp, so a block takes 12 FP64 additions per sum instead of one
// per tree level in every warp (GB300 issues an FP64 warp instruction at 1/64 of the FP32 rate).
// publishing = true: the caller passes the result to publish_and_test_last, whose barrier orders
// warp 0's reads of the shared arrays before the next call's writes; the trailing barrier is skipped.
template <bool GATE>
__device__ Acc block_reduce_check_t(Acc v, bool publishing) {
    __shared__ double part_obj[kBlock];
    __shared__ double part_bnd[kBlock];
    __shared__ double part_sep[GATE ? kBlock : 1];
    __shared__ Acc warp_int[kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    warp_ints(v);
    part_obj[threadIdx.x] = v.obj;
    part_bnd[threadIdx.x] = v.bnd;
    if (GATE) part_sep[threadIdx.x] = v.sep;
    if (lane == 0) warp_int[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double ob = part_obj[lane], bn = part_bnd[lane], sp = GATE ? part_sep[lane] : 0.0;
#pragma unroll
        for (int w = 1; w < kBlock / 32; ++w) {
            ob += part_obj[lane + 32 * w];
            bn += part_bnd[lane + 32 * w];
            if (GATE) sp += part_sep[lane + 32 * w];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ob += shfl_xor(ob, o);
            bn += shfl_xor(bn, o);
            if (GATE) sp += shfl_xor(sp, o);
        }
        Acc w = lane < kBlock / 32 ? warp_int[lane] : acc_identity();
        warp_ints(w);
        v = w;
        v.obj = ob;
        v.bnd = bn;
        v.sep = GATE ? sp : 0.0;
    }
    if (!publishing) __syncthreads();
    return v;
}
__device__ __forceinline__ Acc block_reduce_check(Acc v, bool gate, bool publishing = false) {
    return gate ? block_reduce_check_t<true>(v, publishing) : block_reduce_check_t<false>(v, publishing);
}

__device__ __forceinline__ void store_partial(Partial* p, const Acc& v) {
    p->obj = v.obj; p->bnd = v.bnd; p->sep = v.sep; p->a = v.a;
    p->stat = v.stat; p->prim = v.prim; p->b = v.b; p->hash = v.hash;
    p->n_active = v.nact; p->flags = v.flags; p->pad = 0;
}
__device__ __forceinline__ Acc load_partial(const Partial* p) {
    Acc r;
    r.obj = __ldcg(&p->obj); r.bnd = __ldcg(&p->bnd); r.sep = __ldcg(&p->sep); r.a = __ldcg(&p->a);
    r.stat = __ldcg(reinterpret_cast<const unsigned long long*>(&p->stat));
    r.prim = __ldcg(reinterpret_cast<const unsigned long long*>(&p->prim));
    r.b = __ldcg(reinterpret_cast<const unsigned long long*>(&p->b));
    r.hash = static_cast<unsigned>(__ldcg(reinterpret_cast<const unsigned long long*>(&p->hash)));
    r.nact = static_cast<int>(__ldcg(reinterpret_cast<const long long*>(&p->n_active)));
    r.flags = __ldcg(&p->flags);
    return r;
}

// Publishes the block's partial for tile t and returns true in every thread of the block
// that finished the instance's last outstanding tile.
__device__ bool publish_and_test_last(const View& v, int t, int inst, int ntiles_inst, const Acc& total) {
    __shared__ int is_last;
    if (threadIdx.x == 0) {
        store_partial(&v.partial[t], total);
        __threadfence();
        int prev = atomicAdd(&v.tile_done[inst], 1);
        is_last = (prev == ntiles_inst - 1);
        if (is_last) v.tile_done[inst] = 0;
    }
    __syncthreads();
    bool last = is_last != 0;
    if (last) __threadfence();
    return last;
}

// Reduces the check partials of tiles [tb, te) in a fixed order; valid in thread 0.  Pairs of
// partials are loaded before they are combined (same order, two loads in flight).
template <bool GATE>
__device__ Acc reduce_instance_t(const View& v, int tb, int te) {
    Acc acc = acc_identity();
    int k = tb + static_cast<int>(threadIdx.x);
    for (; k + kBlock < te; k += 2 * kBlock) {
        const Acc p0 = load_partial(&v.partial[k]);
        const Acc p1 = load_partial(&v.partial[k + kBlock]);
        acc = combine_check<GATE>(acc, p0);
        acc = combine_check<GATE>(acc, p1);
    }
    if (k < te) acc = combine_check<GATE>(acc, load_partial(&v.partial[k]));
    return block_reduce_check_t<GATE>(acc, false);
}
__device__ Acc reduce_instance(const View& v, int tb, int te, bool gate) {
    return gate ? reduce_instance_t<true>(v, tb, te) : reduce_instance_t<false>(v, tb, te);
}

// The CG reductions carry two sums (a, obj) and one maximum (b).
// Block sums of a and obj (FP64) and the maximum of b, in a fixed order: every thread's values go
// to shared memory, one warp adds each lane's 8 (thread t: lane t % 32, in order of t), then an
// xor tree over the warp.  GB300 issues an FP64 warp instruction at 1/64 of the FP32 rate whatever
// its active lanes, so this takes 13 FP64 additions per field instead of one per tree level in
// every warp (a lanes-strided layout leaves zeros in the other lanes; adding them is exact).
// `lanes` is kept for the callers' layouts; the maximum reduces over all lanes.
// publishing = true: as for block_reduce_check, the barrier of publish_and_test_last follows.
__device__ Acc block_reduce_ab(Acc v, int lanes = 1, bool warp_data = true, bool publishing = false) {
    (void)lanes;
    __shared__ double part_a[kBlock];
    __shared__ double part_o[kBlock];
    __shared__ unsigned long long part_b[kBlock / 32];
    if (!warp_data) {
        v.a = 0;
        v.obj = 0;
        v.b = 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v.b = umax64(v.b, shfl_xor(v.b, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    part_a[threadIdx.x] = v.a;
    part_o[threadIdx.x] = v.obj;
    if (lane == 0) part_b[warp] = v.b;
    __syncthreads();
    if (warp == 0) {
        double a = part_a[lane], ob = part_o[lane];
#pragma unroll
        for (int w = 1; w < kBlock / 32; ++w) {
            a += part_a[lane + 32 * w];
            ob += part_o[lane + 32 * w];
        }
        unsigned long long b = lane < kBlock / 32 ? part_b[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += shfl_xor(a, o);
            ob += shfl_xor(ob, o);
            b = umax64(b, shfl_xor(b, o));
        }
        v.a = a;
        v.obj = ob;
        v.b = b;
    }
    if (!publishing) __syncthreads();
    return v;
}

// Reduces the CG partials of an instance in a fixed order: the partials of tiles tb, tb + stride,
// ... below te (stride 1: every tile, or every CG work unit's slot).
__device__ Acc reduce_instance_ab(const View& v, int tb, int te, int stride = 1) {
    constexpr int kAhead = 8;
    const int count = (te - tb + stride - 1) / stride;
    Acc acc = acc_identity();
    int i = static_cast<int>(threadIdx.x);
    for (; i + (kAhead - 1) * kBlock < count; i += kAhead * kBlock) {
        double a[kAhead], ob[kAhead];
        unsigned long long b[kAhead];
#pragma unroll
        for (int m = 0; m < kAhead; ++m) {
            const Partial* p = &v.partial[tb + (i + m * kBlock) * stride];
            a[m] = __ldcg(&p->a);
            ob[m] = __ldcg(&p->obj);
            b[m] = __ldcg(reinterpret_cast<const unsigned long long*>(&p->b));
        }
#pragma unroll
        for (int m = 0; m < kAhead; ++m) {
            acc.a += a[m];
            acc.obj += ob[m];
            acc.b = umax64(acc.b, b[m]);
        }
    }
    for (; i < count; i += kBlock) {
        const Partial* p = &v.partial[tb + i * stride];
        acc.a += __ldcg(&p->a);
        acc.obj += __ldcg(&p->obj);
        acc.b = umax64(acc.b, __ldcg(reinterpret_cast<const unsigned long long*>(&p->b)));
    }
    return block_reduce_ab(acc);
}

// ---- one row of check_qp_solution ------------------------------------------------------------
__device__ __forceinline__ unsigned mix_index(unsigned k) {
    k = (k + 1u) * 0x9E3779B9u;
    k ^= k >> 16;
    k *= 0x85EBCA6Bu;
    return k ^ (k >> 13);
}

// One row of check_qp_solution.  The comparisons and finiteness tests run on the bit patterns
// (integer pipes) and the stationarity ratio is divided in FP64 only where it can raise the
// running maximum: this thread's, or `floor`, a maximum other tiles of the same check already
// reached.  The maximum is the one the plain FP64 form gives, bit for bit.
__device__ __forceinline__ void check_row(Acc& a, double xi, double gq, double ci, double li, double ui, double di,
                                          int gate, int row, bool at_lower, bool at_upper,
                                          unsigned long long floor = 0) {
    const uint64_t xb = dbits(xi);
    if (!finite_bits(xb)) {
        a.flags |= 1;
        return;
    }
    a.obj = fma(0.5 * xi, gq, a.obj);
    a.obj = fma(ci, xi, a.obj);
    const double g = gq + ci;
    const uint64_t gb = dbits(g), lb = dbits(li), ub = dbits(ui);
    // |xi - smax(li, smin(ui, xi - g))| with smin(a, b) = b < a ? b : a, smax(a, b) = a < b ? b : a
    const uint64_t tb = dbits(xi - g);
    const uint64_t mb = less_bits(tb, ub) ? tb : ub;
    const uint64_t cb = less_bits(lb, mb) ? mb : lb;
    const double num = fabs(xi - bdouble(cb));
    const uint64_t nb = dbits(num);
    unsigned long long res = 0;  // 0: the ratio leaves the maximum as it is
    if (!finite_bits(gb) || !finite_bits(nb)) {
        res = dbits(kInf);
    } else if (ratio_may_exceed(nb, xb, umax64(a.stat, floor))) {
        const double q = num / (1.0 + fabs(xi));
        res = finite_bits(dbits(q)) ? dbits(q) : dbits(kInf);
    }
    a.stat = umax64(a.stat, res);
    // scaled bound violation, only where the bound is violated (iterates are clamped):
    // li - xi > 0 exactly when xi < li, xi - ui > 0 exactly when ui < xi
    if (less_bits(xb, lb)) a.prim = umax64(a.prim, dbits((li - xi) / (1.0 + fabs(li) + fabs(xi))));
    if (less_bits(ub, xb)) a.prim = umax64(a.prim, dbits((xi - ui) / (1.0 + fabs(ui) + fabs(xi))));
    if ((gb & kAbsMask64) != 0) {  // g != 0 (a NaN included)
        const bool positive = !(gb >> 63) && !nan_bits(gb);
        double target = positive ? li : ui;
        if (finite_bits(dbits(target))) a.bnd += g * (target - xi);
        else a.flags |= 2;
    }
    if (gate) {
        double m = smax(li, smin(ui, -ci / di));
        a.sep += 0.5 * di * m * m + ci * m;
    }
    if (at_lower) {
        a.hash ^= mix_index(2u * static_cast<unsigned>(row));
        a.nact++;
    } else if (at_upper) {
        a.hash ^= mix_index(2u * static_cast<unsigned>(row) + 1u);
        a.nact++;
    }
}

// ---- warp-staged row groups ------------------------------------------------------------------
// A warp takes 32 consecutive rows (one per lane).  Its lanes first form the products of the
// group's nonzeros lane-strided (coalesced value/column loads, up to kWarpBuf independent gathers
// in flight per warp) into a warp-private shared buffer, then each lane sums its own row and
// runs the epilogue with all 32 lanes active.  No block-wide barrier: warps run independently.
// Groups with more than kWarpBuf nonzeros are summed directly, one lane per row.
// Per-warp buffer: 1024 entries of the product type (4 KB for FP32, 8 KB for 8-byte types),
// in dynamic shared memory.
// Buffer entries per warp: 1024 for 4-byte products (4 KB), 768 for 8-byte ones (6 KB).
template <class T>
__host__ __device__ constexpr int warp_entries() { return sizeof(T) == 4 ? 1024 : 768; }
template <class T>
__host__ __device__ constexpr int smem_bytes() { return warp_entries<T>() * static_cast<int>(sizeof(T)) * (kBlock / 32); }
template <class T>
__device__ __forceinline__ T* warp_buffer() {
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    return reinterpret_cast<T*>(dyn_smem) + (threadIdx.x >> 5) * warp_entries<T>();
}

template <class T, class Prod, class Add, class Epi>
__device__ __forceinline__ void warp_groups(const int32_t* __restrict__ rowptr, int rb, int re, T* buf, Prod prod,
                                            Add add, T zero, Epi epi) {
    constexpr int kWarpBuf = warp_entries<T>();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int g = rb + warp * 32; g < re; g += kBlock) {
        const int r = g + lane;
        const bool valid = r < re;
        const int a = valid ? __ldg(rowptr + r) : 0;
        const int b = valid ? __ldg(rowptr + r + 1) : 0;
        const int last = (re - g < 32 ? re - g : 32) - 1;
        const int kb = __shfl_sync(0xffffffffu, a, 0);
        const int ke = __shfl_sync(0xffffffffu, b, last);
        T acc = zero;
        if (ke - kb <= kWarpBuf) {
#pragma unroll 4
            for (int k = kb + lane; k < ke; k += 32) buf[k - kb] = prod(k);
            __syncwarp();
            if (valid)
                for (int k = a; k < b; ++k) acc = add(acc, buf[k - kb]);
            __syncwarp();
        } else if (valid) {
            for (int k = a; k < b; ++k) acc = add(acc, prod(k));
        }
        if (valid) epi(r, acc);
    }
}

// Sub-warp products, full-warp epilogue: a warp takes 32 consecutive rows; in each of LANES passes
// its 32 / LANES sub-groups of LANES lanes form one row sum each (the memory pattern of the tuned
// sub-warp step kernel), and shuffles hand every row sum to its own lane, so the epilogue of the
// 32 rows runs with all 32 lanes active.  Fixed summation order (lane-strided partials, xor tree).
template <int LANES, class T, class Prod, class Add, class Epi>
__device__ __forceinline__ void subwarp_rows(const int32_t* __restrict__ rowptr, int rb, int re, Prod prod, Add add,
                                             T zero, Epi epi) {
    constexpr int R = 32 / LANES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / LANES, sl = lane % LANES;
    for (int base = rb + warp * 32; base < re; base += kBlock) {
        T mine = zero;
#pragma unroll
        for (int pass = 0; pass < LANES; ++pass) {
            const int r = base + pass * R + sub;
            T acc = zero;
            if (r < re) {
                const int ks = __ldg(rowptr + r), ke = __ldg(rowptr + r + 1);
#pragma unroll 4
                for (int k = ks + sl; k < ke; k += LANES) acc = add(acc, prod(k));
            }
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1) acc = add(acc, shfl_xor(acc, o));
            const int g = lane - pass * R;
            const bool mine_now = g >= 0 && g < R;
            const T got = shfl_idx(acc, (mine_now ? g : 0) * LANES);
            if (mine_now) mine = got;
        }
        const int r = base + lane;
        if (r < re) epi(r, mine);
    }
}

// Runs rows [rb, re) with the tile's SpMV structure: sub-warp rows for 1..32 lanes, warp-staged
// rows (shared-memory buffer) for the block- and warp-staged variants.
template <class T, class Prod, class Add, class Epi>
__device__ __forceinline__ void tile_rows(int variant, const int32_t* __restrict__ rowptr, int rb, int re, Prod prod,
                                          Add add, T zero, Epi epi) {
    switch (variant) {
    case 1: subwarp_rows<1, T>(rowptr, rb, re, prod, add, zero, epi); break;
    case 2: subwarp_rows<2, T>(rowptr, rb, re, prod, add, zero, epi); break;
    case 4: subwarp_rows<4, T>(rowptr, rb, re, prod, add, zero, epi); break;
    case 8: subwarp_rows<8, T>(rowptr, rb, re, prod, add, zero, epi); break;
    case 16: subwarp_rows<16, T>(rowptr, rb, re, prod, add, zero, epi); break;
    case 32: subwarp_rows<32, T>(rowptr, rb, re, prod, add, zero, epi); break;
    default: warp_groups<T>(rowptr, rb, re, warp_buffer<T>(), prod, add, zero, epi); break;
    }
}

// FP32 "double-float" arithmetic: an unevaluated pair (hi, lo) carries ~46 significant bits.
// The products of the mixed engine's checks and polish run on the FP32 pipes with it, since
// GB300's FP64 rate is 1/64 of its FP32 rate; FP64 is used once per row.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    return make_float2(s, __fadd_rn(e, __fadd_rn(a.y, b.y)));
}
// (h + l) * x exactly up to the lo-part products: h*x via FMA two-product.
__device__ __forceinline__ float2 df_prod(float h, float l, float x) {
    const float p = __fmul_rn(h, x);
    const float e = __fmaf_rn(h, x, -p);
    return make_float2(p, __fmaf_rn(l, x, e));
}
// (h + l) * (xh + xl)
__device__ __forceinline__ float2 df_prod2(float h, float l, float2 x) {
    const float p = __fmul_rn(h, x.x);
    const float e = __fmaf_rn(h, x.x, -p);
    return make_float2(p, __fmaf_rn(h, x.y, __fmaf_rn(l, x.x, e)));
}
// hi + lo in FP64; the two widenings run in integer arithmetic where both parts are zero or normal
__device__ __forceinline__ double df_value(float2 a) {
    uint64_t h, l;
    if (widen_signed_bits(__float_as_uint(a.x), h) && widen_signed_bits(__float_as_uint(a.y), l))
        return __longlong_as_double(static_cast<long long>(h)) + __longlong_as_double(static_cast<long long>(l));
    return static_cast<double>(a.x) + static_cast<double>(a.y);
}
// The FP32 pair of an FP64 value: hi = RN32(x), lo = RN32(x - hi), in integer arithmetic where
// both are normal floats (split_hilo_bits), with the FP64 conversions elsewhere; the same bits
// either way.
__device__ __forceinline__ float2 df_split(double x) {
    uint32_t h, l;
    if (split_hilo_bits(bits64(x), h, l))
        return make_float2(__uint_as_float(h), __uint_as_float(l));
    const float hf = __double2float_rn(x);
    return make_float2(hf, __double2float_rn(x - static_cast<double>(hf)));
}
// RN32(x), in integer arithmetic where the result is a normal float (round_float_bits); the
// short form for the per-row epilogues, whose values are rarely zero.
__device__ __forceinline__ float rn_float(double x) {
    uint32_t f;
    if (round_float_bits(bits64(x), f)) return __uint_as_float(f);
    return __double2float_rn(x);
}
// RN32(x), RU32(x) and RD32(x) in integer arithmetic (round_dir_bits), zeros and infinities
// included; the FP64 conversion instruction only where the result is subnormal (or x a NaN).
__device__ __forceinline__ float rn_float_all(double x) {
    uint32_t f;
    if (round_dir_bits(bits64(x), 0, f)) return __uint_as_float(f);
    return __double2float_rn(x);
}
__device__ __forceinline__ float ru_float(double x) {
    uint32_t f;
    if (round_dir_bits(bits64(x), 1, f)) return __uint_as_float(f);
    return __double2float_ru(x);
}
__device__ __forceinline__ float rd_float(double x) {
    uint32_t f;
    if (round_dir_bits(bits64(x), -1, f)) return __uint_as_float(f);
    return __double2float_rd(x);
}
// (double)f for a float, in integer arithmetic where f is zero or normal
__device__ __forceinline__ double widen_float(float f) {
    uint64_t d;
    if (widen_signed_bits(__float_as_uint(f), d)) return bdouble(d);
    return static_cast<double>(f);
}

// check_row for the FP32 iterate of the mixed engine: the iterate lies in [l32, u32], a subset of
// [l, u], by construction, so its scaled bound violation is 0; the stationarity ratio is divided
// in FP32 (7 significant digits of the reported residual); sums stay FP64.
__device__ __forceinline__ void check_row_f32(Acc& a, float xf, double gq, double ci, double li, double ui, int row,
                                              bool at_lower, bool at_upper) {
    if (!isfinite(xf)) {
        a.flags |= 1;
        return;
    }
    const double xi = static_cast<double>(xf);
    a.obj = fma(0.5 * xi, gq, a.obj);
    a.obj = fma(ci, xi, a.obj);
    const double g = gq + ci;
    const double num = fabs(xi - smax(li, smin(ui, xi - g)));
    double res = static_cast<double>(__fdiv_rn(static_cast<float>(num), 1.0f + fabsf(xf)));
    if (!isfinite(g) || !isfinite(num)) res = kInf;
    a.stat = umax64(a.stat, dbits(res));
    if (g != 0) {
        double target = g > 0 ? li : ui;
        if (isfinite(target)) a.bnd += g * (target - xi);
        else a.flags |= 2;
    }
    if (at_lower) {
        a.hash ^= mix_index(2u * static_cast<unsigned>(row));
        a.nact++;
    } else if (at_upper) {
        a.hash ^= mix_index(2u * static_cast<unsigned>(row) + 1u);
        a.nact++;
    }
}

// Sources of one check: MODE 0 FP64 values + x64; 1 hi/lo values + x32; 2 hi/lo values + xp.
struct CheckSrc {
    const int32_t* rowptr;
    const int32_t* col;
    const double* val64;
    const float* vhi;
    const float* vlo;
    const double* x64;
    const float* x32;
    const double* xp;
    const float2* xp2;
    const double* c;
    const double* l;
    const double* u;
    const float* l32;
    const float* u32;
    const double* diag;
    int gate;
};

__device__ __forceinline__ double gate_diag(const CheckSrc& s, int r, double fallback) {
    if (!s.gate) return 1.0;
    if (s.diag) return s.diag[r];
    return fallback;
}

// Check of rows [rb, re): accumulates check_row terms into a.
template <int MODE>
__device__ void check_rows(const CheckSrc& s, int variant, int rb, int re, Acc& a, unsigned long long floor = 0) {
    const int32_t* __restrict__ col = s.col;
    if constexpr (MODE == 0) {
        tile_rows<double>(
            variant, s.rowptr, rb, re, [&](int k) { return __ldg(s.val64 + k) * s.x64[__ldg(col + k)]; },
            [](double x, double y) { return x + y; }, 0.0,
            [&](int r, double gq) {
                const double xi = s.x64[r];
                double di = 1.0;
                if (s.gate) {
                    const int ks = __ldg(s.rowptr + r);
                    di = gate_diag(s, r, __ldg(s.rowptr + r + 1) > ks ? __ldg(s.val64 + ks) : 0.0);
                }
                const double li = s.l[r], ui = s.u[r];
                check_row(a, xi, gq, s.c[r], li, ui, di, s.gate, r, less_equal_bits(dbits(xi), dbits(li)),
                          less_equal_bits(dbits(ui), dbits(xi)), floor);
            });
    } else if constexpr (MODE == 1) {
        tile_rows<float2>(
            variant, s.rowptr, rb, re,
            [&](int k) { return df_prod(__ldg(s.vhi + k), __ldg(s.vlo + k), s.x32[__ldg(col + k)]); },
            [](float2 x, float2 y) { return df_add(x, y); }, make_float2(0.f, 0.f),
            [&](int r, float2 acc) {
                const float xf = s.x32[r];
                if (s.gate) {
                    const int ks = __ldg(s.rowptr + r);
                    const double d0 = __ldg(s.rowptr + r + 1) > ks ? static_cast<double>(__ldg(s.vhi + ks)) + __ldg(s.vlo + ks) : 0.0;
                    check_row(a, static_cast<double>(xf), df_value(acc), s.c[r], s.l[r], s.u[r], gate_diag(s, r, d0),
                              1, r, xf <= s.l32[r], xf >= s.u32[r]);
                } else {
                    check_row_f32(a, xf, df_value(acc), s.c[r], s.l[r], s.u[r], r, xf <= s.l32[r], xf >= s.u32[r]);
                }
            });
    } else {
        tile_rows<float2>(
            variant, s.rowptr, rb, re,
            [&](int k) { return df_prod2(__ldg(s.vhi + k), __ldg(s.vlo + k), s.xp2[__ldg(col + k)]); },
            [](float2 x, float2 y) { return df_add(x, y); }, make_float2(0.f, 0.f),
            [&](int r, float2 acc) {
                const double xi = s.xp[r];
                double di = 1.0;
                if (s.gate) {
                    const int ks = __ldg(s.rowptr + r);
                    di = gate_diag(s, r, __ldg(s.rowptr + r + 1) > ks ? static_cast<double>(__ldg(s.vhi + ks)) + __ldg(s.vlo + ks) : 0.0);
                }
                const double li = s.l[r], ui = s.u[r];
                check_row(a, xi, df_value(acc), s.c[r], li, ui, di, s.gate, r, less_equal_bits(dbits(xi), dbits(li)),
                          less_equal_bits(dbits(ui), dbits(xi)), floor);
            });
    }
}

__device__ __forceinline__ CheckSrc source_of(const InstDev& I) {
    CheckSrc s;
    s.rowptr = I.rowptr; s.col = I.col; s.val64 = I.val64; s.vhi = I.vhi; s.vlo = I.vlo;
    s.x64 = I.x64; s.x32 = I.x32; s.xp = I.xp; s.xp2 = I.xp2; s.c = I.c; s.l = I.l; s.u = I.u;
    s.l32 = I.l32; s.u32 = I.u32; s.diag = I.diag; s.gate = I.diag_gate;
    return s;
}

// ---- the state machine after a check (thread 0 of the finalizing block) -------------------
__device__ void fista_betas(InstDev& I, int64_t count) {
    // t_{k+1} = (1 + sqrt(1 + 4 t_k^2)) / 2, beta_k = (t_k - 1) / t_{k+1}
    // (src/accelerated_qp.cpp:47), each operation rounded as the reference's CPU loop rounds it.
    double t = I.t;
    for (int64_t j = 0; j < count; ++j) {
        double nt = __ddiv_rn(__dadd_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(__dmul_rn(4.0, t), t)))), 2.0);
        I.beta[j] = __ddiv_rn(__dsub_rn(t, 1.0), nt);
        I.beta32[j] = static_cast<float>(I.beta[j]);
        t = nt;
    }
    I.t = t;
}

__device__ void finish(InstDev& I, int status, int src) {
    I.status = status;
    I.phase = PH_DONE;
    I.result_src = src;
    I.end_ns = now_ns();
}

__device__ void after_check(InstDev& I, const Acc& tot) {
    const int64_t it_check = I.it_next;
    const int ph = I.phase;
    I.checks++;
    double obj, stat, prim, bound, gap;
    if (tot.flags & 1) {
        obj = __longlong_as_double(0x7ff8000000000000LL);
        stat = kInf; prim = kInf; bound = -kInf; gap = kInf;
    } else {
        obj = tot.obj + I.offset;
        stat = bdouble(tot.stat);
        prim = bdouble(tot.prim);
        if (I.diag_gate) bound = tot.sep + I.offset;
        else bound = (tot.flags & 2) ? -kInf : obj + tot.bnd;
        gap = isfinite(bound) ? fabs(obj - bound) / (1.0 + fabs(obj)) : kInf;
    }
    const double worst = smax(prim, smax(stat, 0.0));
    bool verified = isfinite(obj) && worst <= I.tol;
    if (I.diag_gate) verified = verified && gap <= I.tol;
    I.objective = obj;
    I.primal_res = prim;
    I.stationarity = stat;
    I.dual_bound = bound;
    I.rel_gap = gap;
    I.verified = verified ? 1 : 0;
    I.iterations = it_check;
    const int src = (ph == PH_POLISH_FINISH) ? 2 : (I.precision == PREC_MIXED ? 1 : 0);
    if (verified) { finish(I, ST_OPTIMAL, src); return; }
    if (!isfinite(obj) || !isfinite(stat)) { finish(I, ST_NUMERICAL_ERROR, src); return; }
    if (now_ns() >= I.deadline_ns) { finish(I, ST_TIME_LIMIT, src); return; }
    if (it_check >= I.max_iter) { finish(I, ST_ITERATION_LIMIT, src); return; }
    if (ph == PH_POLISH_FINISH) {
        // The polished point failed verification: the active-set guess was wrong.  FISTA
        // resumes from its own untouched state at it_check.
        I.polish_rounds++;
        I.stable_checks = 0;
    } else if (I.precision == PREC_MIXED && I.polish && I.polish_rounds < 3) {
        const bool stable = tot.hash == I.active_hash && tot.nact == I.n_active;
        I.stable_checks = stable ? I.stable_checks + 1 : 0;
        I.active_hash = tot.hash;
        I.n_active = tot.nact;
        double sw = I.polish_switch;
        for (int k = 0; k < I.polish_rounds; ++k) sw *= 0.1;
        // the chunk's last three iterates share their active set (no move in its last two steps)
        const bool step_stable = it_check - I.it0 >= 2 && I.moved[0] == 0 && I.moved[1] == 0;
        const double step_sw = I.polish_switch > 0 ? sw * (I.step_switch / I.polish_switch) : 0.0;
        if ((I.stable_checks >= 1 && stat <= sw) || (step_stable && stat <= step_sw)) {
            I.phase = PH_POLISH_INIT;
            I.cg_it = 0;
            I.ff_nnz = 0;
            I.ff_rows = 0;
            return;
        }
    }
    I.phase = PH_FISTA;
    I.it0 = it_check;
    I.it_cur = it_check;
    I.moved[0] = 0;
    I.moved[1] = 0;
    I.it_next = it_check + I.interval < I.max_iter ? it_check + I.interval : I.max_iter;
    const int64_t count = I.it_next - I.it0;
    fista_betas(I, count);
    I.fista_iters += count;
}

// ---- step kernel ------------------------------------------------------------------------------
// Active-set motion (mixed precision): in the last two steps of a chunk the step kernel records
// whether any variable entered or left a bound (track = 0 / 1; -1 elsewhere).  A chunk whose last
// three iterates share their active set is "step-stable", which lets the check start the polish
// without waiting for a second check with the same active set.
__device__ __forceinline__ int bound_state(float x, float lo, float up) { return x <= lo ? 1 : (x >= up ? 2 : 0); }
__device__ __forceinline__ void flag_moves(const InstDev& I, int track, bool moved) {
    if (track < 0) return;
    if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) {
        volatile int32_t* f = const_cast<volatile int32_t*>(&I.moved[track]);
        if (*f == 0) *f = 1;
    }
}

// EXACT precision: one thread per row, products and sums rounded separately in column order from
// 0.0 and division by L -- the reference CPU loop's arithmetic exactly.
__device__ void step_rows_exact(const InstDev& I, int rb, int re, int j) {
    const int64_t it = I.it0 + j;
    const int in = static_cast<int>(it & 1), out = in ^ 1;
    const int32_t* __restrict__ rowptr = I.rowptr;
    const int32_t* __restrict__ col = I.col;
    const double* __restrict__ val = I.val64;
    const double* __restrict__ win = I.w64[in];
    double* __restrict__ wout = I.w64[out];
    double* __restrict__ x = I.x64;
    const double* __restrict__ c = I.c;
    const double* __restrict__ l = I.l;
    const double* __restrict__ u = I.u;
    const double beta = I.beta[j];
    const double L = I.L;
    for (int r = rb + static_cast<int>(threadIdx.x); r < re; r += kBlock) {
        double acc = 0.0;
        const int ks = __ldg(rowptr + r), ke = __ldg(rowptr + r + 1);
        for (int k = ks; k < ke; ++k) acc = __dadd_rn(acc, __dmul_rn(__ldg(val + k), __ldg(win + __ldg(col + k))));
        const double v = __dsub_rn(__ldg(win + r), __ddiv_rn(__dadd_rn(acc, __ldg(c + r)), L));
        const double nx = smax(__ldg(l + r), smin(__ldg(u + r), v));
        wout[r] = __dadd_rn(nx, __dmul_rn(beta, __dsub_rn(nx, x[r])));
        x[r] = nx;
    }
}

// FISTA step of rows [rb, re) with warp-staged products: g = Q w, then
// x+ = clip(w - (g + c) / L), w+ = x+ + beta (x+ - x).
template <int PREC>
__device__ void step_rows_staged(const InstDev& I, int rb, int re, int j, int track) {
    const int64_t it = I.it0 + j;
    const int in = static_cast<int>(it & 1), out = in ^ 1;
    const int32_t* __restrict__ col = I.col;
    if constexpr (PREC == PREC_MIXED) {
        const float* __restrict__ val = I.vhi;
        const float* __restrict__ win = I.w32[in];
        float* __restrict__ wout = I.w32[out];
        float* __restrict__ x = I.x32;
        const float* __restrict__ c = I.c32;
        const float* __restrict__ l = I.l32;
        const float* __restrict__ u = I.u32;
        const float beta = I.beta32[j];
        const float* __restrict__ sstep = I.sstep;  // per-row step (preconditioned or 1/L)
        float* buf = warp_buffer<float>();
        bool moved = false;
        warp_groups<float>(
            I.rowptr, rb, re, buf, [&](int k) { return __ldg(val + k) * __ldg(win + __ldg(col + k)); },
            [](float a, float b) { return a + b; }, 0.f,
            [&](int r, float g) {
                const float v = __ldg(win + r) - (g + __ldg(c + r)) * __ldg(sstep + r);
                const float lo = __ldg(l + r), up = __ldg(u + r);
                const float nx = smaxf(lo, sminf(up, v));
                const float xo = x[r];
                wout[r] = nx + beta * (nx - xo);
                x[r] = nx;
                moved |= bound_state(xo, lo, up) != bound_state(nx, lo, up);
            });
        flag_moves(I, track, moved);
    } else {
        const double* __restrict__ val = I.val64;
        const double* __restrict__ win = I.w64[in];
        double* __restrict__ wout = I.w64[out];
        double* __restrict__ x = I.x64;
        const double* __restrict__ c = I.c;
        const double* __restrict__ l = I.l;
        const double* __restrict__ u = I.u;
        const double beta = I.beta[j];
        const double invL = I.invL;
        double* buf = warp_buffer<double>();
        warp_groups<double>(
            I.rowptr, rb, re, buf, [&](int k) { return __ldg(val + k) * __ldg(win + __ldg(col + k)); },
            [](double a, double b) { return a + b; }, 0.0,
            [&](int r, double g) {
                const double v = __ldg(win + r) - (g + __ldg(c + r)) * invL;
                const double nx = smax(__ldg(l + r), smin(__ldg(u + r), v));
                wout[r] = nx + beta * (nx - x[r]);
                x[r] = nx;
            });
    }
}

// Sub-warp rows: LANES lanes per row, a group of 32 / LANES rows per warp pass.
template <int LANES, int PREC>
__device__ void step_rows_subwarp(const InstDev& I, int rb, int re, int j, int track) {
    using T = typename std::conditional<PREC == PREC_MIXED, float, double>::type;
    const int64_t it = I.it0 + j;
    const int in = static_cast<int>(it & 1), out = in ^ 1;
    constexpr int RPW = 32 / LANES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / LANES, sl = lane % LANES;
    const int32_t* __restrict__ rowptr = I.rowptr;
    const int32_t* __restrict__ col = I.col;
    const T* __restrict__ val;
    const T* __restrict__ win;
    T* __restrict__ wout;
    T* __restrict__ x;
    const T* __restrict__ c;
    const T* __restrict__ l;
    const T* __restrict__ u;
    T beta, invL;
    if constexpr (PREC == PREC_MIXED) {
        val = I.vhi; win = I.w32[in]; wout = I.w32[out]; x = I.x32; c = I.c32; l = I.l32; u = I.u32;
        beta = I.beta32[j]; invL = I.invLf;
    } else {
        val = I.val64; win = I.w64[in]; wout = I.w64[out]; x = I.x64; c = I.c; l = I.l; u = I.u;
        beta = I.beta[j]; invL = I.invL;
    }
    const float* __restrict__ sstep = I.sstep;
    bool moved = false;
    for (int base = rb + warp * RPW; base < re; base += (kBlock / 32) * RPW) {
        const int r = base + sub;
        T acc = 0;
        if (r < re) {
            const int ks = __ldg(rowptr + r), ke = __ldg(rowptr + r + 1);
#pragma unroll 4
            for (int k = ks + sl; k < ke; k += LANES) acc += __ldg(val + k) * __ldg(win + __ldg(col + k));
        }
        acc = group_sum<LANES>(acc);
        if (r < re && sl == 0) {
            T step;
            if constexpr (PREC == PREC_MIXED) step = __ldg(sstep + r);  // per-row step
            else step = invL;
            const T v = __ldg(win + r) - (acc + __ldg(c + r)) * step;
            const T lo = __ldg(l + r), up = __ldg(u + r);
            const T nx = (lo < ((up < v) ? up : v)) ? ((up < v) ? up : v) : lo;
            const T xo = x[r];
            wout[r] = nx + beta * (nx - xo);
            x[r] = nx;
            if constexpr (PREC == PREC_MIXED) moved |= bound_state(xo, lo, up) != bound_state(nx, lo, up);
        }
    }
    if constexpr (PREC == PREC_MIXED) flag_moves(I, track, moved);
}

// Block-staged tile (nnz <= kTileNnz): the tile's products are formed by all threads at once
// (kTileNnz / kBlock independent gathers per thread), then one thread per row sums and updates.
template <int PREC>
__device__ void step_tile_block(const InstDev& I, int rb, int re, int j, int track) {
    using T = typename std::conditional<PREC == PREC_MIXED, float, double>::type;
    extern __shared__ __align__(16) unsigned char dyn_smem[];
    T* prod = reinterpret_cast<T*>(dyn_smem);
    const int64_t it = I.it0 + j;
    const int in = static_cast<int>(it & 1), out = in ^ 1;
    const int32_t* __restrict__ rowptr = I.rowptr;
    const int kb = __ldg(rowptr + rb), ke = __ldg(rowptr + re);
    const int cnt = ke - kb;
    const int32_t* __restrict__ cl = I.col + kb;
    const T* __restrict__ val;
    const T* __restrict__ win;
    T* __restrict__ wout;
    T* __restrict__ x;
    const T* __restrict__ c;
    const T* __restrict__ l;
    const T* __restrict__ u;
    T beta, invL;
    if constexpr (PREC == PREC_MIXED) {
        val = I.vhi + kb; win = I.w32[in]; wout = I.w32[out]; x = I.x32; c = I.c32; l = I.l32; u = I.u32;
        beta = I.beta32[j]; invL = I.invLf;
    } else {
        val = I.val64 + kb; win = I.w64[in]; wout = I.w64[out]; x = I.x64; c = I.c; l = I.l; u = I.u;
        beta = I.beta[j]; invL = I.invL;
    }
    const float* __restrict__ sstep = I.sstep;
#pragma unroll 8
    for (int k = threadIdx.x; k < cnt; k += kBlock) prod[k] = __ldg(val + k) * __ldg(win + __ldg(cl + k));
    __syncthreads();
    bool moved = false;
    for (int r = rb + static_cast<int>(threadIdx.x); r < re; r += kBlock) {
        const int a = __ldg(rowptr + r) - kb, b = __ldg(rowptr + r + 1) - kb;
        T acc = 0;
        for (int k = a; k < b; ++k) acc += prod[k];
        T step;
        if constexpr (PREC == PREC_MIXED) step = __ldg(sstep + r);  // per-row step
        else step = invL;
        const T v = __ldg(win + r) - (acc + __ldg(c + r)) * step;
        const T lo = __ldg(l + r), up = __ldg(u + r);
        const T nx = (lo < ((up < v) ? up : v)) ? ((up < v) ? up : v) : lo;
        const T xo = x[r];
        wout[r] = nx + beta * (nx - xo);
        x[r] = nx;
        if constexpr (PREC == PREC_MIXED) moved |= bound_state(xo, lo, up) != bound_state(nx, lo, up);
    }
    if constexpr (PREC == PREC_MIXED) flag_moves(I, track, moved);
    __syncthreads();  // prod is reused by the next tile
}

// One tile of FISTA step j0 of a body (iteration it_cur + j0 of an instance whose chunk is not
// done) with a fixed SpMV structure.  The test is uniform over the block.
template <int PREC, int VAR>
__device__ __forceinline__ void step_tile(const View& v, const Tile& T, int j0) {
    const InstDev& I = v.inst[T.inst];
    if (I.status != ST_RUNNING || I.phase != PH_FISTA || I.precision != PREC) return;
    const int64_t it = I.it_cur + j0;
    if (it >= I.it_next) return;
    const int j = static_cast<int>(it - I.it0);  // position in the chunk
    const int count = static_cast<int>(I.it_next - I.it0);
    const int track = (PREC == PREC_MIXED && count >= 2 && j >= count - 2) ? j - (count - 2) : -1;
    if constexpr (PREC == PREC_FP64_EXACT) {
        step_rows_exact(I, T.row_begin, T.row_end, j);
    } else if constexpr (VAR == VAR_TILE) {
        if (__ldg(I.rowptr + T.row_end) - __ldg(I.rowptr + T.row_begin) <= kTileNnz)
            step_tile_block<PREC>(I, T.row_begin, T.row_end, j, track);
        else
            step_rows_staged<PREC>(I, T.row_begin, T.row_end, j, track);
    } else if constexpr (VAR == VAR_WARP) {
        step_rows_staged<PREC>(I, T.row_begin, T.row_end, j, track);
    } else {
        step_rows_subwarp<VAR, PREC>(I, T.row_begin, T.row_end, j, track);
    }
}

// Step kernel of one group (precision, SpMV structure): grid-stride over the group's tiles.
// The sub-warp structures of 2 to 32 lanes per row run 6 blocks per SM (40 registers; measured
// on the 1M random graph, 4 lanes: 85.9 us per step against 94.5 us at the compiler's 48
// registers and 89.9 us at 8 blocks); one lane per row and the staged structures keep the
// compiler's choice (the 1M tridiagonal and grid steps are faster there).
template <int VAR>
constexpr int step_min_blocks() { return (VAR == VAR_TILE || VAR == VAR_WARP || VAR == 1) ? 0 : 6; }

template <int PREC, int VAR>
__global__ void __launch_bounds__(kBlock, step_min_blocks<VAR>()) step_kernel(View v, int group, int j0) {
    if (j0 >= v.ctrl->step_due[PREC]) return;  // every chunk of this precision ends before step j0
    const int b = v.ctrl->group_begin[group], e = v.ctrl->group_begin[group + 1];
    for (int t = b + static_cast<int>(blockIdx.x); t < e; t += gridDim.x) step_tile<PREC, VAR>(v, v.tiles[v.group_tiles[t]], j0);
}

// FP64_EXACT engine: one structure, every tile of the table (other precisions skip).
__global__ void __launch_bounds__(kBlock) step_exact_kernel(View v, int j0) {
    if (j0 >= v.ctrl->step_due[PREC_FP64_EXACT]) return;
    const int nt = v.ctrl->n_tiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) step_tile<PREC_FP64_EXACT, 1>(v, v.tiles[t], j0);
}

// ---- check kernel -----------------------------------------------------------------------------
// One kernel per precision family (FAMILY_MIXED: FP32 iterate or polished point; FAMILY_FP64:
// fp64 and fp64_exact), so each carries only its own check path and its own register budget.
constexpr int FAMILY_FP64 = 0;
constexpr int FAMILY_MIXED = 1;    // FP32 iterate of the mixed engine (FISTA phase)
constexpr int FAMILY_VERIFY = 2;   // polished point of the mixed engine (once per polish)

template <int FAMILY>
__global__ void __launch_bounds__(kBlock, 3) check_kernel(View v) {
    if (v.ctrl->check_due[FAMILY] == 0) return;  // no instance due for this family in this body
    const int nt = v.ctrl->n_tiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const Tile T = v.tiles[t];
        InstDev& I = v.inst[T.inst];
        if (I.status != ST_RUNNING) continue;
        if (I.phase == PH_FISTA && I.it_cur < I.it_next) continue;  // chunk still running
        if ((I.precision == PREC_MIXED) != (FAMILY != FAMILY_FP64)) continue;
        const int ph = I.phase;
        if (FAMILY == FAMILY_VERIFY ? ph != PH_POLISH_FINISH : ph != PH_FISTA) continue;
        const CheckSrc s = source_of(I);
        // the largest stationarity ratio earlier tiles of this check reached
        const unsigned long long floor = __ldcg(&I.stat_floor);
        Acc a = acc_identity();
        // the mixed checks sum double-float products (eight FP32 additions each), so they take
        // sub-warp rows of a few lanes (the CG product's choice, about two entries per lane)
        // rather than the step's structure: on the 1M random graph the verification with 2 / 4 /
        // 8 / 16 lanes or the step's warp-staged rows measured 2.004 / 2.016 / 2.027 / 2.083 /
        // 2.047 ms per solve
        if constexpr (FAMILY == FAMILY_VERIFY) check_rows<2>(s, I.lanes_cg, T.row_begin, T.row_end, a, floor);
        else if constexpr (FAMILY == FAMILY_MIXED) check_rows<1>(s, I.lanes_cg, T.row_begin, T.row_end, a);
        else check_rows<0>(s, T.variant, T.row_begin, T.row_end, a, floor);
        Acc total = block_reduce_check(a, s.gate != 0, true);
        // raised before this tile's partial is published, so before the finalizer resets it
        if (threadIdx.x == 0 && total.stat > floor) atomicMax(&I.stat_floor, total.stat);
        const int2 R = v.ranges[T.inst];
        if (publish_and_test_last(v, t, T.inst, R.y - R.x, total)) {
            Acc inst_total = reduce_instance(v, R.x, R.y, s.gate != 0);
            if (threadIdx.x == 0) {
                after_check(I, inst_total);
                I.stat_floor = 0;  // the next check starts from nothing
            }
            __syncthreads();
        }
    }
}

// ---- FP64 free-set polish ---------------------------------------------------------------------
// Solves Q_FF x_F = -c_F - Q_FA x_A by Jacobi-preconditioned conjugate gradients, the free set F
// being the variables the FP32 iterate holds strictly inside its bounds.  Vectors are FP64; the
// matrix products are formed in FP32 double-float arithmetic from the hi/lo values and the FP32
// pairs xp2 / p2 kept beside xp / p.
// polish_init lists each tile's free rows in ascending order at free_rows[row_begin ...], their
// count at free_cnt[tile index within the instance] and each free row's list position (row_begin
// + its index) in pos_of[row] and xq[row].z, -1 for the rows held at a bound; the CG vectors (r,
// z, p, s, q, p2, xf) live on those positions, and the packed Q_FF's columns are positions too (an
// instance's tiling depends on the instance alone, so the positions survive changes of the batch).
// CG stopping measure |r| / (1 + |x|) of one row, in FP32 (it is compared with half the
// tolerance), as the bit pattern of a non-negative float: maxima reduce on the integer pipes, and
// r and x are rounded to FP32 in integer arithmetic (the FP64 pipe runs at 1/64 of the FP32 rate
// on this GPU).
__device__ __forceinline__ unsigned long long cg_ratio_bits(double r, double x) {
    const float ratio = __fdividef(fabsf(rn_float(r)), 1.0f + fabsf(rn_float(x)));
    return static_cast<unsigned long long>(__float_as_uint(ratio));
}

__device__ __forceinline__ bool polish_phase(const InstDev& I, int phase) {
    return I.status == ST_RUNNING && I.phase == phase;
}

__global__ void __launch_bounds__(kBlock) polish_init_kernel(View v) {
    __shared__ int warp_free[kBlock / 32];
    const int nt = v.ctrl->n_tiles;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const Tile T = v.tiles[t];
        const InstDev& I = v.inst[T.inst];
        if (!polish_phase(I, PH_POLISH_INIT)) continue;
        const float* __restrict__ x32 = I.x32;
        const float* __restrict__ l32 = I.l32;
        const float* __restrict__ u32 = I.u32;
        const double* __restrict__ l = I.l;
        const double* __restrict__ u = I.u;
        double* __restrict__ xp = I.xp;
        float2* __restrict__ xp2 = I.xp2;
        int4* __restrict__ xq = I.xq;
        int32_t* __restrict__ pos_out = I.pos_of;
        int32_t* __restrict__ list = I.free_rows + T.row_begin;
        int count = 0;
        for (int r0 = T.row_begin; r0 < T.row_end; r0 += kBlock) {
            const int r = r0 + static_cast<int>(threadIdx.x);
            bool is_free = false;
            float2 x2 = make_float2(0.f, 0.f);
            if (r < T.row_end) {
                const float xf = x32[r];
                double xv;
                if (xf <= l32[r]) xv = l[r];
                else if (xf >= u32[r]) xv = u[r];
                else { xv = static_cast<double>(xf); is_free = true; }
                x2 = df_split(xv);
                xp[r] = xv;
                xp2[r] = x2;
            }
            const unsigned m = __ballot_sync(0xffffffffu, is_free);
            if (lane == 0) warp_free[warp] = __popc(m);
            __syncthreads();
            int before = count, total = count;
#pragma unroll
            for (int w = 0; w < kBlock / 32; ++w) {
                before += w < warp ? warp_free[w] : 0;
                total += warp_free[w];
            }
            if (r < T.row_end) {
                const int j = before + __popc(m & ((1u << lane) - 1u));
                if (is_free) list[j] = r;
                const int pos = is_free ? T.row_begin + j : -1;
                xq[r] = make_int4(__float_as_int(x2.x), __float_as_int(x2.y), pos, 0);
                pos_out[r] = pos;
            }
            __syncthreads();
            count = total;
        }
        if (threadIdx.x == 0) I.free_cnt[t - v.ranges[T.inst].x] = count;
    }
}

// Polish products over a tile's free-row list, LANES lanes per row (chosen from the average row
// length at admission): the warps of the block take the list in turns of 32 / LANES
// rows, so a tile's few hundred free rows spread evenly over the block, and the leading lane of
// each group runs the row's epilogue.  Per row: lane-strided partial sums, then an xor tree.

// Residual pass: r = -(Q xp + c) over the full rows (xq holds the snapped point's pairs), and the
// tile's Q_FF entries (free rows, free columns; p is zero on the fixed rows, so the omitted
// entries contribute nothing to the CG products) packed densely from the start of the tile's
// extent: a first pass counts each free row's kept entries, a block scan places the rows, and
// the product pass writes them in column order.
template <int LANES>
__device__ void count_kept(const InstDev& I, const int32_t* __restrict__ list, int n, int32_t* kept_of) {
    constexpr int R = 32 / LANES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / LANES, sl = lane % LANES;
    const int32_t* __restrict__ rowptr = I.rowptr;
    const int32_t* __restrict__ col = I.col;
    const int32_t* __restrict__ pos_of = I.pos_of;
    for (int g = warp; g * R < n; g += kBlock / 32) {  // warp-uniform
        const int j = g * R + sub;
        int cnt = 0;
        if (j < n) {
            const int r = list[j];
            const int ks = __ldg(rowptr + r), ke = __ldg(rowptr + r + 1);
#pragma unroll 4
            for (int k = ks + sl; k < ke; k += LANES) cnt += pos_of[__ldg(col + k)] >= 0 ? 1 : 0;
        }
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (sl == 0 && j < n) kept_of[j] = cnt;
    }
}

// Exclusive prefix sum of v[0..n) in place (n <= kTileRows), block-wide; returns the total.
__device__ int block_exclusive_scan(int32_t* v, int n) {
    __shared__ int warp_tot[kBlock / 32];
    __shared__ int total;
    constexpr int kPer = kTileRows / kBlock;  // entries per thread
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int mine[kPer], sum = 0;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int idx = threadIdx.x * kPer + i;
        mine[i] = idx < n ? v[idx] : 0;
        sum += mine[i];
    }
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += warp_tot[w];
    if (threadIdx.x == kBlock - 1) total = before + incl;
    int run = before + incl - sum;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int idx = threadIdx.x * kPer + i;
        if (idx < n) v[idx] = run;
        run += mine[i];
    }
    __syncthreads();
    return total;
}

template <int LANES>
__device__ void residual_rows(const InstDev& I, const int32_t* __restrict__ list, int n, int base,
                              const int32_t* __restrict__ start_of, float2* rowsum, float2* coupling, Acc& a) {
    constexpr int R = 32 / LANES;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / LANES, sl = lane % LANES;
    const unsigned group = (LANES == 32 ? 0xffffffffu : ((1u << LANES) - 1u)) << (sub * LANES);
    const unsigned below = (1u << lane) - 1u;
    const int32_t* __restrict__ rowptr = I.rowptr;
    const int32_t* __restrict__ col = I.col;
    const float* __restrict__ vhi = I.vhi;
    const float* __restrict__ vlo = I.vlo;
    const int4* __restrict__ xq = I.xq;
    int32_t* __restrict__ col_ff = I.col_ff;
    float* __restrict__ hi_ff = I.hi_ff;
    float* __restrict__ lo_ff = I.lo_ff;
    // the packed row's entry count and start, at its position in the tile's free list (the CG
    // product reads them without first loading the row index)
    int32_t* __restrict__ cnt_ff = I.cnt_ff + (list - I.free_rows);
    int32_t* __restrict__ start_ff = I.start_ff + (list - I.free_rows);
    for (int g = warp; g * R < n; g += kBlock / 32) {  // warp-uniform
        const int j = g * R + sub;
        int r = -1, ks = 0, len = 0, dst = 0;
        if (j < n) {
            r = list[j];
            ks = __ldg(rowptr + r);
            len = __ldg(rowptr + r + 1) - ks;
            dst = base + start_of[j];
        }
        const int wmax = __reduce_max_sync(0xffffffffu, len);
        float2 acc = make_float2(0.f, 0.f);
        float2 e_next = make_float2(0.f, 0.f);  // Q(r, r + 1), the coupling to the adjacent row
        int kept = 0;
        for (int i = 0; i < wmax; i += LANES) {  // warp-uniform
            const bool valid = i + sl < len;
            bool keep = false;
            int cc = 0, pc = -1;
            float h = 0.f, lo = 0.f;
            if (valid) {
                const int k = ks + i + sl;
                cc = __ldg(col + k);
                h = __ldg(vhi + k);
                lo = __ldg(vlo + k);
                const int4 q = xq[cc];  // the column's pair and position in one gather
                acc = df_add(acc, df_prod2(h, lo, make_float2(__int_as_float(q.x), __int_as_float(q.y))));
                pc = q.z;
                keep = pc >= 0;
                if (cc == r + 1) e_next = make_float2(e_next.x + h, e_next.y + lo);
            }
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (keep) {
                const int pos = dst + kept + __popc(m & group & below);
                col_ff[pos] = pc;  // the column's free-list position
                hi_ff[pos] = h;
                lo_ff[pos] = lo;
            }
            kept += __popc(m & group);
        }
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) {
            acc = df_add(acc, shfl_xor(acc, o));
            e_next.x += __shfl_xor_sync(0xffffffffu, e_next.x, o);
            e_next.y += __shfl_xor_sync(0xffffffffu, e_next.y, o);
        }
        if (sl == 0 && r >= 0) {
            cnt_ff[j] = kept;
            start_ff[j] = dst;
            rowsum[j] = acc;
            coupling[j] = e_next;
        }
    }
}

// The residual pass's FP64 epilogue over a tile's free rows (list positions t < n, after a block
// barrier): r = -(Q xp + c), the preconditioned z = M^-1 r, p = z, s = 0, and the CG reduction's
// r.z and max |r|/(1+|x|).  M is the polish's preconditioner: the tridiagonal part of Q_FF within
// the tile, Q(r, r + 1) between free rows adjacent in the list and in Q, kept only where both
// rows stay strictly diagonally dominant with their couplings (so every pivot of the chain's
// LDL' factorization is positive and M is positive definite) and cut every kChain list positions
// (so a tile's long runs split over several threads); a row without kept couplings is a Jacobi row
// (1/Q_rr).  On the tridiagonal family M is Q_FF within runs of up to kChain free rows, on the
// grid it couples the free runs of each grid row (line relaxation), on a random graph it is the
// Jacobi preconditioner.  A tile without chains runs the Jacobi rows alone (pc_tile 0: the vector
// step's single pass); otherwise each chain is factored and solved in shared memory by one thread
// in FP32 (Thomas recurrence: pivots m_0 = Q_00, m_i = Q_ii - e_{i-1}^2 / m_{i-1}), and 1/m and the
// kept coupling (FP32 values) are stored per list position for the vector step.  FP32 chains took
// the tridiagonal family from 1.33 to 1.22 ms per solve (residual pass 252 -> 166 us, vector step
// 65 -> 48 us cold; CG 6 -> 7 iterations).
// Chain cap, measured on the tridiagonal family (every variable free, 1M rows; FP64 chains):
// 16 / 32 / 64 / 128 / 256 / 512 positions: 2.09 / 1.69 / 1.44 / 1.47 / 2.01 / 3.08 ms per solve
// (15 / 10 / 6 / 4 / 4 / 4 CG iterations): longer chains precondition better but solve sequentially.
constexpr int kChain = 64;
constexpr int kChainMin = 8;

// Sum of one int per thread over the block (every thread gets the total); block-wide barriers.
__device__ int block_sum_int(int v) {
    __shared__ int part[kBlock / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    int total = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) total += part[w];
    return total;
}

__device__ void residual_epilogue(const InstDev& I, const int32_t* __restrict__ list, int n, int tile,
                                  const float2* rowsum, const float2* coupling, Acc& a) {
    __shared__ double res[kTileRows];  // r per list position
    __shared__ double dg[kTileRows];   // Q_rr per list position
    __shared__ double ec[kTileRows];   // coupling to the next position; then the forward values
    __shared__ double ek[kTileRows];   // kept coupling
    __shared__ double zs[kTileRows];   // z of the chain rows
    const double* __restrict__ c = I.c;
    const double* __restrict__ dinv = I.dinv;
    const double* __restrict__ diag = I.diag;
    const double* __restrict__ xp = I.xp;
    const int q0 = static_cast<int>(list - I.free_rows);  // list position t is q0 + t
    double* __restrict__ r_out = I.r + q0;
    double* __restrict__ z_out = I.z + q0;
    double* __restrict__ p_out = I.p + q0;
    double* __restrict__ s_out = I.s + q0;
    double* __restrict__ xf_out = I.xf + q0;
    float2* __restrict__ p2_out = I.p2 + q0;
    double* __restrict__ pc_inv = I.pc_inv + q0;
    double* __restrict__ pc_e = I.pc_e + q0;
    // the CG start on list position t (row r): r, z = M^-1 r, p = z, s = 0 and x
    auto row_out = [&](int t, int r, double rr, double zz) {
        const double xr = xp[r];
        a.a = fma(rr, zz, a.a);
        a.b = umax64(a.b, cg_ratio_bits(rr, xr));
        r_out[t] = rr;
        z_out[t] = zz;
        p_out[t] = zz;
        s_out[t] = 0.0;
        p2_out[t] = df_split(zz);
        xf_out[t] = xr;
    };
    bool any = false;
    for (int t = threadIdx.x; t < n; t += kBlock) {
        const int r = list[t];
        res[t] = -(df_value(rowsum[t]) + c[r]);
        double e = 0.0;
        if (t + 1 < n && list[t + 1] == r + 1 && (t + 1) % kChain != 0)
            e = static_cast<double>(coupling[t].x) + coupling[t].y;
        ec[t] = e;
        if (e != 0.0) {
            any = true;
            dg[t] = diag[r];
        }
        if (t > 0 && list[t - 1] == r - 1) dg[t] = diag[r];  // a possible chain row's pivot source
    }
    bool chains = __syncthreads_or(any) != 0;
    if (chains) {
        bool kept_any = false;
        for (int t = threadIdx.x; t < n; t += kBlock) {
            const double e = ec[t];
            bool keep = false;
            if (e != 0.0) {
                const double left = t > 0 ? fabs(ec[t - 1]) : 0.0;
                keep = left + fabs(e) < dg[t] && fabs(e) + fabs(ec[t + 1]) < dg[t + 1];
            }
            ek[t] = keep ? e : 0.0;
            kept_any |= keep;
        }
        chains = __syncthreads_or(kept_any) != 0;
        if (chains) {
            // chains pay for their sequential solves only when they are long: a tile keeps them
            // when its chained rows average kChainMin or more per chain.  Measured on the 1024^2
            // grid (free runs of about 2.5 rows, 3.7 among chained rows): chains took CG from 24
            // to 19 iterations but the vector step from 21 to 45 us, 1.90 -> 2.15 ms per solve,
            // and tiles averaging 4 or more still cost 2.06 ms; on the tridiagonal family (every
            // variable free, chains at the kChain cap) CG falls from 78 to 6 iterations.
            int in_chain = 0, heads = 0;
            for (int t = threadIdx.x; t < n; t += kBlock) {
                const bool left = t > 0 && ek[t - 1] != 0.0;
                if (ek[t] != 0.0 || left) ++in_chain;
                if (ek[t] != 0.0 && !left) ++heads;
            }
            const int rows_in_chains = block_sum_int(in_chain);
            const int n_chains = block_sum_int(heads);
            chains = rows_in_chains >= kChainMin * n_chains;
        }
    }
    if (threadIdx.x == 0) I.pc_tile[tile] = chains ? 1 : 0;
    if (!chains) {
        for (int t = threadIdx.x; t < n; t += kBlock) {
            const int r = list[t];
            const double inv = dinv[r];
            pc_inv[t] = inv;  // the vector step's Jacobi rows read 1 / Q_rr by position
            row_out(t, r, res[t], res[t] * inv);
        }
        return;
    }
    // chains of two or more rows, one thread each, in shared memory; the chains are numbered
    // densely so that consecutive lanes take them; each chain's arithmetic does not depend on
    // which thread runs it.  The factorization and the solves run in FP32: M only preconditions
    // (CG's recurrences and the verification stay FP64), a chain's recurrence is sequential, and
    // an FP32 step is about a tenth of an FP64 one on this GPU.  The shared arrays of the
    // dominance test are reused as FP32 arrays (dg: Q_rr and r; ec: forward values and 1/pivot;
    // zs: z and the kept couplings).
    __shared__ int32_t starts[kTileRows / 2];
    __shared__ int n_starts;
    float* dgf = reinterpret_cast<float*>(dg);
    float* rsf = dgf + kTileRows;
    float* yf = reinterpret_cast<float*>(ec);
    float* ivf = yf + kTileRows;
    float* zf = reinterpret_cast<float*>(zs);
    float* ekf = zf + kTileRows;
    double dv[kTileRows / kBlock], rv[kTileRows / kBlock];
#pragma unroll
    for (int q = 0; q < kTileRows / kBlock; ++q) {
        const int t = threadIdx.x + q * kBlock;
        dv[q] = t < n ? dg[t] : 0.0;
        rv[q] = t < n ? res[t] : 0.0;
    }
    if (threadIdx.x == 0) n_starts = 0;
    __syncthreads();  // every FP64 Q_rr read before the FP32 views overwrite it
#pragma unroll
    for (int q = 0; q < kTileRows / kBlock; ++q) {
        const int t = threadIdx.x + q * kBlock;
        if (t < n) {
            dgf[t] = rn_float_all(dv[q]);
            rsf[t] = rn_float_all(rv[q]);
            const float e = rn_float_all(ek[t]);
            ekf[t] = e;
            // a chain starts where an FP32 coupling follows none (a coupling below FP32's range
            // ends a chain, as it does in the vector step)
            if (e != 0.0f && (t == 0 || rn_float_all(ek[t - 1]) == 0.0f)) starts[atomicAdd(&n_starts, 1)] = t;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < n_starts; k += kBlock) {
        const int t = starts[k];
        int end = t;
        while (ekf[end] != 0.0f) ++end;  // ek[n - 1] == 0
        float iv = __frcp_rn(dgf[t]);
        float y = rsf[t] * iv;
        ivf[t] = iv;
        yf[t] = y;
        for (int i = t + 1; i <= end; ++i) {
            float e = ekf[i - 1];
            // pivot m_i = Q_ii - e^2 / m_{i-1}; strict dominance keeps it above the row's margin in
            // exact arithmetic, and where FP32 rounding would eat a margin below 2^-20 Q_ii the
            // chain is cut here instead (the coupling dropped, the same in the vector step)
            float m = __fmaf_rn(-e, e * iv, dgf[i]);
            if (!(m > dgf[i] * 0x1p-20f)) {
                m = dgf[i];
                e = 0.0f;
                ekf[i - 1] = 0.0f;
            }
            iv = __frcp_rn(m);
            y = (rsf[i] - e * y) * iv;
            ivf[i] = iv;
            yf[i] = y;
        }
        float z = yf[end];
        zf[end] = z;
        for (int i = end - 1; i >= t; --i) {
            z = yf[i] - ekf[i] * ivf[i] * z;
            zf[i] = z;
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += kBlock) {
        const int r = list[t];
        // the rows the chain phase wrote
        const bool in_chain = rn_float_all(ek[t]) != 0.0f || (t > 0 && rn_float_all(ek[t - 1]) != 0.0f);
        double zz;
        if (in_chain) {
            zz = widen_float(zf[t]);
            pc_inv[t] = widen_float(ivf[t]);
            pc_e[t] = widen_float(ekf[t]);
        } else {  // a Jacobi row
            const double inv = dinv[r];
            pc_inv[t] = inv;
            pc_e[t] = 0.0;
            zz = res[t] * inv;
        }
        row_out(t, r, res[t], zz);
    }
}

// CG product w = Q_FF u over one work unit, the free rows of up to kCgUnitMax consecutive tiles of
// one instance taken as one list (position p of the unit: tile k with pre[k] <= p < pre[k + 1],
// row j = p - pre[k] of that tile's free list), u gathered from its FP32 pairs; accumulates
// gamma = r.u, delta = w.u and max |r|/(1+|x|) (the single reduction of the Chronopoulos-Gear form
// of preconditioned CG).  LANES lanes per row for the products, kCgGroups row groups of a warp
// with their loads in flight together, then the FP64 epilogue one row per thread on full warps.
__device__ __forceinline__ int unit_tile(const int* pre, int nk, int p) {
    int k = 0;
#pragma unroll
    for (int i = 1; i < kCgUnitMax; ++i) k += (i < nk && p >= pre[i]) ? 1 : 0;
    return k;
}

// The unit's free-row table in shared memory: pre[k] (prefix of the tiles' free counts, the
// total at pre[kCgUnitMax]) and rbeg[k] (the tile's first row, where its free list starts).  The
// caller's previous readers of the table are past a block barrier.
__device__ __forceinline__ void unit_table(const View& v, const InstDev& I, int t0, int first_tile, int nk, int* pre,
                                          int* rbeg) {
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nk; ++k) {
            pre[k] = acc;
            rbeg[k] = v.tiles[t0 + k].row_begin;
            acc += I.free_cnt[t0 - first_tile + k];
        }
        for (int k = nk; k <= kCgUnitMax; ++k) pre[k] = acc;
    }
    __syncthreads();
}

template <int LANES>
__device__ void matvec_unit(const InstDev& I, const int* pre, const int* rbeg, int nk, int total, float2* rowsum,
                            Acc& a) {
    constexpr int R = 32 / LANES;
    constexpr int W = kBlock / 32;
    constexpr int U = kCgGroups;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int sub = lane / LANES, sl = lane % LANES;
    const int32_t* __restrict__ col = I.col_ff;
    const float* __restrict__ vhi = I.hi_ff;
    const float* __restrict__ vlo = I.lo_ff;
    const int32_t* __restrict__ cnt = I.cnt_ff;
    const int32_t* __restrict__ start = I.start_ff;
    const float2* __restrict__ p2 = I.p2;  // u as FP32 pairs
    const double* __restrict__ u = I.z;
    const double* __restrict__ rr_v = I.r;
    const double* __restrict__ xf = I.xf;
    double* __restrict__ q_out = I.q;      // w
    const int groups = (total + R - 1) / R;
    for (int g0 = warp; g0 < groups; g0 += W * U) {  // warp-uniform
        int ks[U], ke[U];
#pragma unroll
        for (int m = 0; m < U; ++m) {
            const int p = (g0 + m * W) * R + sub;
            ks[m] = 0;
            ke[m] = 0;
            if (p < total) {
                const int k = unit_tile(pre, nk, p);
                const int at = rbeg[k] + (p - pre[k]);
                ks[m] = start[at];
                ke[m] = ks[m] + cnt[at];
            }
        }
        int longest = 0;
#pragma unroll
        for (int m = 0; m < U; ++m) longest = max(longest, ke[m] - ks[m]);
        float2 acc[U];
#pragma unroll
        for (int m = 0; m < U; ++m) acc[m] = make_float2(0.f, 0.f);
        // kCgUnroll entries of each row group per lane per pass: every load of the pass (entries,
        // then gathers) is issued before the first product; the sums keep the per-lane order
        for (int i = sl; i < longest; i += LANES * kCgUnroll) {
            int c[U][kCgUnroll];
            float h[U][kCgUnroll], l[U][kCgUnroll];
            float2 xv[U][kCgUnroll];
#pragma unroll
            for (int m = 0; m < U; ++m) {
#pragma unroll
                for (int q = 0; q < kCgUnroll; ++q) {
                    const int e = ks[m] + i + q * LANES;
                    const bool in = e < ke[m];
                    c[m][q] = in ? __ldg(col + e) : -1;
                    h[m][q] = in ? __ldg(vhi + e) : 0.f;
                    l[m][q] = in ? __ldg(vlo + e) : 0.f;
                }
            }
#pragma unroll
            for (int m = 0; m < U; ++m) {
#pragma unroll
                for (int q = 0; q < kCgUnroll; ++q) xv[m][q] = c[m][q] >= 0 ? p2[c[m][q]] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int m = 0; m < U; ++m) {
#pragma unroll
                for (int q = 0; q < kCgUnroll; ++q)
                    if (c[m][q] >= 0) acc[m] = df_add(acc[m], df_prod2(h[m][q], l[m][q], xv[m][q]));
            }
        }
#pragma unroll
        for (int m = 0; m < U; ++m) {
#pragma unroll
            for (int o = LANES / 2; o > 0; o >>= 1) acc[m] = df_add(acc[m], shfl_xor(acc[m], o));
            const int p = (g0 + m * W) * R + sub;
            if (sl == 0 && p < total) rowsum[p] = acc[m];
        }
    }
    // the FP64 epilogue, one free row per thread on full warps, kCgUnroll rows per pass with
    // their loads issued together; each thread adds its rows in ascending order
    __syncthreads();
    for (int p0 = threadIdx.x; p0 < total; p0 += kBlock * kCgUnroll) {
        int r[kCgUnroll];  // list positions
        double ui[kCgUnroll], ri[kCgUnroll], xi[kCgUnroll];
#pragma unroll
        for (int q = 0; q < kCgUnroll; ++q) {
            const int p = p0 + q * kBlock;
            r[q] = -1;
            if (p < total) {
                const int k = unit_tile(pre, nk, p);
                r[q] = rbeg[k] + (p - pre[k]);
            }
        }
#pragma unroll
        for (int q = 0; q < kCgUnroll; ++q) {
            ui[q] = r[q] >= 0 ? u[r[q]] : 0.0;
            ri[q] = r[q] >= 0 ? rr_v[r[q]] : 0.0;
            xi[q] = r[q] >= 0 ? xf[r[q]] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < kCgUnroll; ++q) {
            if (r[q] < 0) continue;
            const double w = df_value(rowsum[p0 + q * kBlock]);
            q_out[r[q]] = w;
            a.a = fma(ri[q], ui[q], a.a);
            a.obj = fma(w, ui[q], a.obj);
            a.b = umax64(a.b, cg_ratio_bits(ri[q], xi[q]));
        }
    }
}

template <int LANES>
__device__ int residual_tile(const InstDev& I, const int32_t* list, int n_free, int base, int32_t* start_of,
                             float2* rowsum, float2* coupling, Acc& a) {
    count_kept<LANES>(I, list, n_free, start_of);
    __syncthreads();
    const int kept = block_exclusive_scan(start_of, n_free);
    residual_rows<LANES>(I, list, n_free, base, start_of, rowsum, coupling, a);
    return kept;
}

// Residual (with the packing of Q_FF) over tile rows [rb, ...) of one instance (its tile index
// `tile` within the instance); returns the tile's packed Q_FF entries.
__device__ int polish_rows(const InstDev& I, int rb, int tile, int n_free, Acc& a) {
    __shared__ int32_t start_of[kTileRows];  // free-list positions of the packed rows
    __shared__ float2 rowsum[kTileRows];     // row sums handed to the FP64 epilogue
    __shared__ float2 coupling[kTileRows];   // Q(r, r + 1) of each free row (hi, lo)
    const int32_t* list = I.free_rows + rb;
    const int base = __ldg(I.rowptr + rb);
    int kept;
    switch (I.lanes_res) {
    case 1: kept = residual_tile<1>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    case 2: kept = residual_tile<2>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    case 4: kept = residual_tile<4>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    case 8: kept = residual_tile<8>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    case 16: kept = residual_tile<16>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    default: kept = residual_tile<32>(I, list, n_free, base, start_of, rowsum, coupling, a); break;
    }
    // the FP64 epilogue, one free row (or one chain of rows) per thread on full warps
    __syncthreads();
    residual_epilogue(I, list, n_free, tile, rowsum, coupling, a);
    return kept;
}

// Four blocks per SM (64 registers, a few spills): 2.307 ms per 1M random-graph solve against
// 2.329 ms at the compiler's three (80 registers); the check kernels measured slower at four.
// Over the CG product's work units (runs of consecutive tiles of one instance, as many as the
// resident blocks): one unit per block in one round, the unit's tiles one after the other, one
// reduction and one publication per unit (the unit's partial in its instance's slot R.x + index).
__global__ void __launch_bounds__(kBlock, 4) polish_residual_kernel(View v) {
    const int nu = v.ctrl->n_units;
    for (int un = blockIdx.x; un < nu; un += gridDim.x) {
        const int4 U = v.units[un];  // first tile, tiles, index and units of its instance
        const Tile T0 = v.tiles[U.x];
        InstDev& I = v.inst[T0.inst];
        if (!polish_phase(I, PH_POLISH_INIT)) continue;
        const int2 R = v.ranges[T0.inst];
        Acc a = acc_identity();
        int kept = 0, n_free_unit = 0;
        for (int q = 0; q < U.y; ++q) {
            const int t = U.x + q;
            if (q > 0) __syncthreads();  // the previous tile's shared arrays have been read
            const int n_free = I.free_cnt[t - R.x];
            kept += polish_rows(I, v.tiles[t].row_begin, t - R.x, n_free, a);
            n_free_unit += n_free;
        }
        if (threadIdx.x == 0) {  // Q_FF size of this polish round, for the byte accounting
            atomicAdd(reinterpret_cast<unsigned long long*>(&I.ff_nnz), static_cast<unsigned long long>(kept));
            atomicAdd(reinterpret_cast<unsigned long long*>(&I.ff_rows), static_cast<unsigned long long>(n_free_unit));
        }
        Acc total = block_reduce_ab(a, I.lanes_res, true, true);
        if (publish_and_test_last(v, R.x + U.z, T0.inst, U.w, total)) {
            Acc inst_total = reduce_instance_ab(v, R.x, R.x + U.w);
            if (threadIdx.x == 0) {
                // residual pass: the full CSR (hi/lo values + columns) and row pointers, xq (the
                // snapped point's pairs and the positions, gathered) and c; the packed Q_FF
                // written (hi/lo + column) with its row starts and counts; r, z, p, s, p2, x and
                // the preconditioner's 1/pivot written and 1/diag read on the free rows
                const double nnz = static_cast<double>(__ldg(I.rowptr + I.n));
                const double N = static_cast<double>(I.n);
                const double fz = static_cast<double>(I.ff_nnz), fr = static_cast<double>(I.ff_rows);
                I.polish_bytes += 12.0 * nnz + 4.0 * (N + 1) + 24.0 * N + 12.0 * fz + 8.0 * fr + 64.0 * fr;
                I.rz = inst_total.a;
                I.cg_res = static_cast<double>(__uint_as_float(static_cast<unsigned>(inst_total.b)));
                I.cg_it = 0;
                I.phase = (I.cg_res <= I.cg_tol || !(I.rz > 0)) ? PH_POLISH_FINISH : PH_POLISH_CG;
                if (I.phase == PH_POLISH_FINISH) atomicSub(&v.ctrl->n_cg, 1);
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(kBlock, 4) cg_matvec_kernel(View v) {
    __shared__ int pre[kCgUnitMax + 1];
    __shared__ int rbeg[kCgUnitMax];
    __shared__ float2 rowsum[kCgRowsum];
    const int nu = v.ctrl->n_units;
    for (int un = blockIdx.x; un < nu; un += gridDim.x) {
        const int4 U = v.units[un];  // first tile, tiles, index and units of its instance
        const int t0 = U.x;
        const Tile T = v.tiles[t0];
        InstDev& I = v.inst[T.inst];
        if (!polish_phase(I, PH_POLISH_CG)) continue;
        const int2 R = v.ranges[T.inst];
        const int nk = U.y;
        unit_table(v, I, t0, R.x, nk, pre, rbeg);
        const int total = pre[kCgUnitMax];
        Acc a = acc_identity();
        switch (I.lanes_cg) {
        case 1: matvec_unit<1>(I, pre, rbeg, nk, total, rowsum, a); break;
        case 2: matvec_unit<2>(I, pre, rbeg, nk, total, rowsum, a); break;
        case 4: matvec_unit<4>(I, pre, rbeg, nk, total, rowsum, a); break;
        case 8: matvec_unit<8>(I, pre, rbeg, nk, total, rowsum, a); break;
        case 16: matvec_unit<16>(I, pre, rbeg, nk, total, rowsum, a); break;
        default: matvec_unit<32>(I, pre, rbeg, nk, total, rowsum, a); break;
        }
        Acc tot = block_reduce_ab(a, I.lanes_cg, true, true);
        // the unit's partial in slot R.x + index: the instance's partials are contiguous
        if (publish_and_test_last(v, R.x + U.z, T.inst, U.w, tot)) {
            Acc inst_total = reduce_instance_ab(v, R.x, R.x + U.w);
            if (threadIdx.x == 0) {
                // Chronopoulos-Gear: gamma_i = r_i.u_i, delta_i = (Q u_i).u_i, beta_i =
                // gamma_i / gamma_{i-1}, alpha_i = gamma_i / (delta_i - beta_i gamma_i / alpha_{i-1})
                const double gamma = inst_total.a, delta = inst_total.obj;
                I.cg_res = static_cast<double>(__uint_as_float(static_cast<unsigned>(inst_total.b)));
                const bool first = I.cg_it == 0;
                I.cg_it++;
                I.cg_total++;
                // one CG iteration on Q_FF: its packed entries (hi/lo + column), and per free
                // row the product's 48 bytes and the vector step's 104 (bqp_profile_cg)
                I.polish_bytes += 12.0 * static_cast<double>(I.ff_nnz) + 152.0 * static_cast<double>(I.ff_rows);
                bool stop = I.cg_res <= I.cg_tol || I.cg_it > I.cg_max || !isfinite(gamma) || !isfinite(delta);
                if (!stop) {
                    const double beta = first ? 0.0 : gamma / I.rz;
                    const double den = first ? delta : delta - beta * gamma / I.alpha;
                    const double alpha = gamma / den;
                    if (alpha > 0 && isfinite(alpha)) {
                        I.alpha = alpha;
                        I.beta_cg = beta;
                        I.rz = gamma;
                    } else {
                        stop = true;  // breakdown
                    }
                }
                if (stop) {
                    I.phase = PH_POLISH_FINISH;
                    atomicSub(&v.ctrl->n_cg, 1);
                }
            }
            __syncthreads();
        }
    }
}

// CG vector step on the free-list positions: p = u + beta p, s = w + beta s, x += alpha p,
// r -= alpha s, u = M^-1 r (and its FP32 pairs for the next product), every vector streamed by
// position.  No reduction: the product kernel's finalizer already chose alpha and beta.  Instances
// that finished CG write x back to their free rows, snapped into the box, here.
// In a graph, block 0 also decides whether the CG loop runs another iteration: while an instance
// still iterates and fewer than `cap` iterations ran (the product kernel, which completed before
// this launch, counted finishing instances down).
__global__ void __launch_bounds__(kBlock) cg_vector_kernel(View v, cudaGraphConditionalHandle h_cg, int cap) {
    if (cap > 0 && blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* ctrl = v.ctrl;
        const int it = ++ctrl->cg_iters;
        ctrl->kernels += 2;
        cudaGraphSetConditional(h_cg, (ctrl->n_cg > 0 && it < cap) ? 1u : 0u);
    }

    const int nt = v.ctrl->n_tiles;
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const Tile T = v.tiles[t];
        const InstDev& I = v.inst[T.inst];
        if (I.status != ST_RUNNING) continue;
        if (I.phase == PH_POLISH_CG) {
            const double alpha = I.alpha, beta = I.beta_cg;
            const int tile = t - v.ranges[T.inst].x;
            const int n_free = I.free_cnt[tile];
            const int q0 = T.row_begin;  // free row j of the tile is list position q0 + j
            const double* __restrict__ w = I.q + q0;
            double* __restrict__ u = I.z + q0;
            double* __restrict__ p = I.p + q0;
            double* __restrict__ s = I.s + q0;
            double* __restrict__ xf = I.xf + q0;
            double* __restrict__ rr_v = I.r + q0;
            float2* __restrict__ u2 = I.p2 + q0;
            const double* __restrict__ pc_inv = I.pc_inv + q0;
            if (!I.pc_tile[tile]) {  // Jacobi rows only: u = r / Q_rr
                for (int j = static_cast<int>(threadIdx.x); j < n_free; j += kBlock) {
                    const double pn = fma(beta, p[j], u[j]);
                    const double sn = fma(beta, s[j], w[j]);
                    const double rn = fma(-alpha, sn, rr_v[j]);
                    const double un = rn * pc_inv[j];
                    p[j] = pn;
                    s[j] = sn;
                    xf[j] = fma(alpha, pn, xf[j]);
                    rr_v[j] = rn;
                    u[j] = un;
                    u2[j] = df_split(un);
                }
            } else {
                // the residual pass's chains (pc_e links a position to the next): the updates
                // first; then the Jacobi rows in parallel (FP64) and one thread per chain (the
                // chains numbered densely; the recurrence in FP32 from the FP32 factors the
                // residual pass stored), in shared memory; then the stores of u
                __shared__ double rs[kTileRows];
                __shared__ double ys[kTileRows];
                __shared__ double pi[kTileRows];
                __shared__ float rsf[kTileRows];
                __shared__ float pif[kTileRows];
                __shared__ float pef[kTileRows];
                __shared__ float yf[kTileRows];
                __shared__ int32_t starts[kTileRows / 2];
                __shared__ int n_starts_s;
                int* n_starts = &n_starts_s;
                if (threadIdx.x == 0) n_starts_s = 0;
                const double* __restrict__ pc_e = I.pc_e + q0;
                for (int j = static_cast<int>(threadIdx.x); j < n_free; j += kBlock) {
                    const double pn = fma(beta, p[j], u[j]);
                    const double sn = fma(beta, s[j], w[j]);
                    const double rn = fma(-alpha, sn, rr_v[j]);
                    const double iv = pc_inv[j];
                    p[j] = pn;
                    s[j] = sn;
                    xf[j] = fma(alpha, pn, xf[j]);
                    rr_v[j] = rn;
                    rs[j] = rn;
                    pi[j] = iv;
                    rsf[j] = rn_float_all(rn);
                    pif[j] = rn_float_all(iv);         // exact on chain rows (stored from FP32)
                    pef[j] = rn_float_all(pc_e[j]);    // exact: FP32 couplings or 0
                }
                __syncthreads();
                for (int j = static_cast<int>(threadIdx.x); j < n_free; j += kBlock) {
                    const bool linked_left = j > 0 && pef[j - 1] != 0.0f;
                    if (pef[j] == 0.0f && !linked_left) ys[j] = rs[j] * pi[j];  // a Jacobi row
                    else if (!linked_left) starts[atomicAdd(n_starts, 1)] = j;
                }
                __syncthreads();
                const int chains = *n_starts;
                for (int k = static_cast<int>(threadIdx.x); k < chains; k += kBlock) {
                    const int j = starts[k];
                    float y = rsf[j] * pif[j];
                    yf[j] = y;
                    int end = j;
                    while (pef[end] != 0.0f) {
                        ++end;
                        y = (rsf[end] - pef[end - 1] * y) * pif[end];
                        yf[end] = y;
                    }
                    float un = y;
                    for (int i = end - 1; i >= j; --i) {
                        un = yf[i] - pef[i] * pif[i] * un;
                        yf[i] = un;
                    }
                }
                __syncthreads();
                for (int j = static_cast<int>(threadIdx.x); j < n_free; j += kBlock) {
                    const bool in_chain = pef[j] != 0.0f || (j > 0 && pef[j - 1] != 0.0f);
                    if (in_chain) {
                        u[j] = widen_float(yf[j]);
                        u2[j] = make_float2(yf[j], 0.0f);
                    } else {
                        u[j] = ys[j];
                        u2[j] = df_split(ys[j]);
                    }
                }
                __syncthreads();  // the shared arrays are reused by the block's next chain tile
            }
        } else if (I.phase == PH_POLISH_FINISH) {
            // x of the free rows back from the list positions, snapped into the box (the rows
            // held at a bound kept their bound from polish_init); repeating it changes nothing
            const int n_free = I.free_cnt[t - v.ranges[T.inst].x];
            const int32_t* __restrict__ list = I.free_rows + T.row_begin;
            const double* __restrict__ xf = I.xf + T.row_begin;
            const double* __restrict__ l = I.l;
            const double* __restrict__ uu = I.u;
            double* __restrict__ xp = I.xp;
            float2* __restrict__ xp2 = I.xp2;
            for (int j = static_cast<int>(threadIdx.x); j < n_free; j += kBlock) {
                const int r = list[j];
                const double xv = smax(l[r], smin(uu[r], xf[j]));
                xp[r] = xv;
                xp2[r] = df_split(xv);
            }
        }
    }
}

// ---- control kernels (one block) ---------------------------------------------------------------
struct Counts {
    int running, fista[3], polish;
    int check_due[3];  // per check family: FP64 engines, the mixed FP32 iterate, the polished point
    int step_due[3];   // per precision: the longest remaining chunk among FISTA instances (capped by steps)
};

// steps > 0: also the step launches with work per precision (a chunk needs it_next - it_cur more)
__device__ Counts count_phases(const View& v, bool mirror, int steps = 0) {
    __shared__ int s[11];
    if (threadIdx.x < 11) s[threadIdx.x] = 0;
    __syncthreads();
    int nr = 0, nf[3] = {0, 0, 0}, np = 0, due[3] = {0, 0, 0}, need[3] = {0, 0, 0};
    const int n = v.ctrl->n_inst;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const InstDev& I = v.inst[i];
        const int st = I.status;
        if (mirror) v.status_mirror[i] = st;
        if (st != ST_RUNNING) continue;
        nr++;
        const int pk = I.precision == PREC_MIXED ? 1 : I.precision == PREC_FP64_EXACT ? 2 : 0;
        if (I.phase == PH_FISTA) {
            nf[pk]++;
            if (I.it_cur >= I.it_next) due[pk == 1 ? 1 : 0]++;  // the check kernel's test
            else if (steps > 0) {
                const int64_t left = I.it_next - I.it_cur;
                need[pk] = max(need[pk], left < steps ? static_cast<int>(left) : steps);
            }
        } else if (I.phase == PH_POLISH_INIT || I.phase == PH_POLISH_CG) {
            np++;
        } else if (I.phase == PH_POLISH_FINISH && pk == 1) {
            due[2]++;
        }
    }
    if (nr) atomicAdd(&s[0], nr);
    for (int k = 0; k < 3; ++k) {
        if (nf[k]) atomicAdd(&s[1 + k], nf[k]);
        if (due[k]) atomicAdd(&s[5 + k], due[k]);
        if (need[k]) atomicMax(&s[8 + k], need[k]);
    }
    if (np) atomicAdd(&s[4], np);
    __syncthreads();
    Counts c;
    c.running = s[0];
    for (int k = 0; k < 3; ++k) {
        c.fista[k] = s[1 + k];
        c.check_due[k] = s[5 + k];
        c.step_due[k] = s[8 + k];
    }
    c.polish = s[4];
    return c;
}

// End of a body: every instance that stepped in it (FISTA phase) advances by the steps it ran.
// A mixed solve whose chunk just completed step-stable (no variable crossed a bound in its last
// two steps) goes straight to its first polish attempt, without the check of the FP32 iterate:
// the polished point is verified in FP64 anyway, and a failed attempt resumes FISTA from this
// iterate through the checked path.
__device__ void advance_chunks(const View& v, int steps) {
    const int n = v.ctrl->n_inst;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        InstDev& I = v.inst[i];
        if (I.status != ST_RUNNING || I.phase != PH_FISTA) continue;
        const int64_t to = I.it_cur + steps;
        I.it_cur = to < I.it_next ? to : I.it_next;
        if (I.it_cur == I.it_next && I.precision == PREC_MIXED && I.polish && I.polish_rounds == 0 &&
            I.step_switch > 0 && I.it_next - I.it0 >= 2 && I.it_next < I.max_iter && I.moved[0] == 0 &&
            I.moved[1] == 0) {
            I.phase = PH_POLISH_INIT;
            I.cg_it = 0;
            I.ff_nnz = 0;
            I.ff_rows = 0;
            I.stable_checks = 0;
            I.iterations = I.it_next;
        }
    }
    __syncthreads();
}

// The polish branch runs polish_init and the residual, then a CG loop whose iterations the
// direction kernel counts into Ctrl::kernels.
__global__ void gate_kernel(View v, cudaGraphConditionalHandle h_fp64, cudaGraphConditionalHandle h_mixed,
                            cudaGraphConditionalHandle h_exact, cudaGraphConditionalHandle h_polish,
                            cudaGraphConditionalHandle h_cg, StepLaunches steps, int body_steps) {
    const Counts c = count_phases(v, false, body_steps);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            v.ctrl->n_fista[k] = c.fista[k];
            v.ctrl->step_due[k] = c.step_due[k];
        }
        v.ctrl->n_polish = c.polish;
        v.ctrl->n_cg = c.polish;
        v.ctrl->cg_iters = 0;
        long long launched = 4;  // three check kernels + gate
        for (int k = 0; k < 3; ++k) launched += c.fista[k] > 0 ? steps.n[k] : 0;
        launched += c.polish > 0 ? 2 : 0;
        v.ctrl->kernels += launched;
        cudaGraphSetConditional(h_fp64, c.fista[0] > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_mixed, c.fista[1] > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_exact, c.fista[2] > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_polish, c.polish > 0 ? 1u : 0u);
        cudaGraphSetConditional(h_cg, c.polish > 0 ? 1u : 0u);
    }
}

__global__ void control_kernel(View v, cudaGraphConditionalHandle loop_h, int steps) {
    advance_chunks(v, steps);
    const Counts c = count_phases(v, true);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) v.ctrl->check_due[k] = c.check_due[k];
        Ctrl* ctrl = v.ctrl;
        ctrl->bodies++;
        ctrl->kernels += 1;
        ctrl->running = c.running;
        cudaGraphSetConditional(loop_h, (c.running > 0 && ctrl->bodies < ctrl->body_cap) ? 1u : 0u);
    }
}

__global__ void gate_plain_kernel(View v, int steps) {
    const Counts c = count_phases(v, false, steps);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) {
            v.ctrl->n_fista[k] = c.fista[k];
            v.ctrl->step_due[k] = c.step_due[k];
        }
        v.ctrl->n_polish = c.polish;
        v.ctrl->n_cg = c.polish;
        v.ctrl->cg_iters = 0;
    }
}

__global__ void control_plain_kernel(View v, int steps) {
    advance_chunks(v, steps);
    const Counts c = count_phases(v, true);
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; ++k) v.ctrl->check_due[k] = c.check_due[k];
        v.ctrl->bodies++;
        v.ctrl->running = c.running;
    }
}

// x0 = clip(0, l, u) and w = x0 for row r (the pointers of a record do not change on re-arming).
__device__ __forceinline__ void init_row(const InstDev& I, int r) {
    if (I.precision == PREC_MIXED) {
        const float x0 = smaxf(I.l32[r], sminf(I.u32[r], 0.0f));
        I.x32[r] = x0;
        I.w32[0][r] = x0;
    } else {
        const double x0 = smax(I.l[r], smin(I.u[r], 0.0));
        I.x64[r] = x0;
        I.w64[0][r] = x0;
    }
}

// Start of a solve: clock, deadline and (mixed) the first chunk.  One thread.
__device__ void start_instance(InstDev& I) {
        const int64_t start = now_ns();
        I.start_ns = start;
        I.deadline_ns = start + I.deadline_ns;  // host stores the budget in nanoseconds
        I.end_ns = 0;
        if (I.arm_chunk) {
            // mixed precision: x0 = clip(0) is not checked; the first chunk of steps is armed here
            // as a check of x0 would arm it.  With a short interval the first chunk is one and a
            // half intervals long: the active set still moves in the first steps, so a check
            // there could not start the polish.
            I.it0 = 0;
            I.it_cur = 0;
            I.moved[0] = 0;
            I.moved[1] = 0;
            const int64_t first = I.interval <= 16 ? I.interval + I.interval / 2 : I.interval;
            I.it_next = first < I.max_iter ? first : I.max_iter;
            fista_betas(I, I.it_next);
            I.fista_iters += I.it_next;
        }
}

__global__ void init_instance_kernel(View v, int slot, int n) {
    InstDev& I = v.inst[slot];
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) init_row(I, r);
    if (blockIdx.x == 0 && threadIdx.x == 0) start_instance(I);
}

// Re-arms a list of resident solves in one launch.  Block b takes rows [span.y, span.y + kRearmRows)
// of staged record span.x; the block holding row 0 also installs the record in its slot and
// starts the solve.
__global__ void __launch_bounds__(kBlock) rearm_kernel(View v, const InstDev* __restrict__ stage,
                                                       const int32_t* __restrict__ slots, const int2* __restrict__ spans) {
    const int2 sp = spans[blockIdx.x];
    const InstDev& S = stage[sp.x];
    const int end = S.n < sp.y + kRearmRows ? S.n : sp.y + kRearmRows;
    for (int r = sp.y + static_cast<int>(threadIdx.x); r < end; r += kBlock) init_row(S, r);
    if (sp.y == 0) {
        InstDev& I = v.inst[slots[sp.x]];
        const uint4* src = reinterpret_cast<const uint4*>(&S);
        uint4* dst = reinterpret_cast<uint4*>(&I);
        for (int w = threadIdx.x; w < static_cast<int>(sizeof(InstDev) / 16); w += kBlock) dst[w] = src[w];
        __syncthreads();
        if (threadIdx.x == 0) {
            // the power estimate replaces the host's Gershgorin L (the mixed engine's steps
            // already carry it in sstep; its L is then the estimate for the matrix they scale)
            if (I.lip_device) {
                I.L = *I.lprec;
                I.invL = 1.0 / I.L;
                I.invLf = static_cast<float>(I.invL);
            }
            start_instance(I);
        }
    }
}

// The Gershgorin bound the gate found (admission kernels that run after it read L from there).
__device__ __forceinline__ double gate_lipschitz(const InstDev& I) {
    return __longlong_as_double(static_cast<long long>(I.gate->lip_bits));
}

// ---- admission pass over the nonzeros: convexity gate, Gershgorin bound, diagonal, hi/lo split -----
// Per row, the row's entries in column order (the order of the reference's Gershgorin sum,
// src/accelerated_qp.cpp:25-26, so L comes out bit for bit): sum |Q_ik| in FP64, the diagonal
// Q_ii (duplicate diagonal entries summed) and the off-diagonal radius sum_{j != i} |Q_ij|; a row
// with Q_ii < 0, or Q_ii = 0 beside off-diagonal entries, is indefinite, and one with
// Q_ii < radius breaks diagonal dominance (check_convex_hessian, src/qp_admm.cpp:30-39).  The same
// pass stores the FP64 diagonal (the Jacobi preconditioner and the diagonal dual-gap gate; a
// single diagonal entry is stored as given) and, for the mixed engine, the hi/lo FP32 values.
// FP64 instructions run at 1/64 of the FP32 rate on GB300 and cost the same whatever a warp's
// active lanes, so the pass keeps them off the nonzeros:
//   * the split runs in integer arithmetic (split_hilo_bits);
//   * both sums are bracketed by FP32 sums rounded down and up of the FP32 bounds of |Q_ij|
//     (abs_bounds_bits).  By induction over the row, RD32(lo + rd) <= RD64(s + |q|) <=
//     fl64(s + |q|) and the same upward, so the FP64 column-order sum lies in its bracket;
//   * Q_ii < lo and Q_ii >= hi decide dominance as the FP64 radius would; a row whose diagonal
//     falls inside the bracket sums its radius in FP64;
//   * L is the largest FP64 row sum, and only a row whose upper bound reaches the largest lower
//     bound of any row can hold it: the pass keeps that floor in the result (an atomic maximum,
//     read back by each warp per group of rows) and sums in FP64 only the rows at or above it.
//     The row with the largest sum is always among them, so L is the same bits whatever the
//     order in which the warps run.
// A warp takes 32 consecutive rows and walks their entries in windows of kGateBuf: it stages a
// window's values and columns in shared memory with coalesced loads (writing the split as it
// goes), and each lane then adds the part of its own row inside the window, so every row's sums
// run in column order whatever its length; the FP64 sums re-read their rows (from L2).
constexpr int kGateWarps = 4;      // warps per block of the gate kernel
constexpr int kGateBuf = 512;      // staged entries per warp (6 KB: values and columns)

__global__ void __launch_bounds__(kGateWarps * 32) convexity_gate_kernel(const int32_t* __restrict__ rowptr,
                                                                          const int32_t* __restrict__ col,
                                                                          const double* __restrict__ val, int n,
                                                                          GateResult* out, double* __restrict__ diag,
                                                                          float* __restrict__ vhi,
                                                                          float* __restrict__ vlo) {
    __shared__ uint64_t sval[kGateWarps][kGateBuf];  // the values' bit patterns
    __shared__ int32_t scol[kGateWarps][kGateBuf];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t* bv = sval[warp];
    int32_t* bc = scol[warp];
    const unsigned long long* __restrict__ vbits = reinterpret_cast<const unsigned long long*>(val);
    unsigned long long best = 0, floor_seen = 0;
    int indefinite = 0, nondominant = 0, flags = 0;
    const int groups = (n + 31) / 32;
    for (int g = blockIdx.x * kGateWarps + warp; g < groups; g += gridDim.x * kGateWarps) {  // warp-uniform
        const int r = g * 32 + lane;
        const bool valid = r < n;
        const int a = valid ? __ldg(rowptr + r) : 0;
        const int b = valid ? __ldg(rowptr + r + 1) : 0;
        const int last = min(n - g * 32, 32) - 1;
        const int kb = __shfl_sync(0xffffffffu, a, 0);
        const int ke = __shfl_sync(0xffffffffu, b, last);
        float sum_lo = 0.0f, sum_hi = 0.0f, rad_lo = 0.0f, rad_hi = 0.0f;
        int nd = 0, kd = 0;  // diagonal entries of the row and the first one's position
        bool offd = false;   // a nonzero off-diagonal value (check_qp_solution's positive_diagonal)
        for (int w = kb; w < ke; w += kGateBuf) {
            const int we = min(ke, w + kGateBuf);
            // the window's loads first, several per lane in flight; then the entry work from
            // shared memory
#pragma unroll 4
            for (int k = w + lane; k < we; k += 32) {
                bv[k - w] = __ldg(vbits + k);
                bc[k - w] = __ldg(col + k);
            }
            __syncwarp();
            for (int k = w + lane; k < we; k += 32) {
                const uint64_t vb = bv[k - w];
                const int32_t c = bc[k - w];
                if (static_cast<uint32_t>(c) >= static_cast<uint32_t>(n) ||
                    (vb & 0x7ff0000000000000ull) == 0x7ff0000000000000ull)
                    flags |= kGateInvalid;
                if (vb << 1) flags |= kGateNonzero;
                if (vhi) {
                    uint32_t h, l;
                    if (!split_hilo_bits(vb, h, l)) {
                        const double v = __longlong_as_double(static_cast<long long>(vb));
                        const float hf = __double2float_rn(v);
                        h = __float_as_uint(hf);
                        l = __float_as_uint(__double2float_rn(v - static_cast<double>(hf)));
                    }
                    vhi[k] = __uint_as_float(h);
                    vlo[k] = __uint_as_float(l);
                }
            }
            __syncwarp();
            const int ka = max(a, w), kz = valid ? min(b, we) : ka;
            for (int k = ka - w; k < kz - w; ++k) {
                const uint64_t mag = bv[k] & 0x7fffffffffffffffull;
                uint32_t lo, hi;
                abs_bounds_bits(mag, lo, hi);
                sum_lo = __fadd_rd(sum_lo, __uint_as_float(lo));
                sum_hi = __fadd_ru(sum_hi, __uint_as_float(hi));
                if (bc[k] == r) {
                    if (nd++ == 0) kd = k + w;
                } else {
                    rad_lo = __fadd_rd(rad_lo, __uint_as_float(lo));
                    rad_hi = __fadd_ru(rad_hi, __uint_as_float(hi));
                    if (mag) offd = true;
                }
            }
            __syncwarp();
        }
        // the floor: the largest lower bound of a row sum, this group's and the others' so far
        unsigned long long group_floor = valid ? widen_bits(__float_as_uint(sum_lo)) : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) group_floor = umax64(group_floor, shfl_xor(group_floor, o));
        if (group_floor > floor_seen) {
            if (lane == 0) atomicMax(&out->floor_bits, group_floor);
            floor_seen = group_floor;
        }
        floor_seen = umax64(floor_seen, *reinterpret_cast<volatile unsigned long long*>(&out->floor_bits));
        if (valid) {
            // Q_ii: a single diagonal entry as given, duplicates summed in column order from 0
            double d = 0.0;
            if (nd == 1) {
                d = __ldg(val + kd);
            } else if (nd > 1) {
                for (int k = kd; k < b; ++k)
                    if (__ldg(col + k) == r) d += __ldg(val + k);
            }
            if (widen_bits(__float_as_uint(sum_hi)) >= floor_seen) {
                double total = 0.0;
                for (int k = a; k < b; ++k) total += fabs(__ldg(val + k));
                best = umax64(best, dbits(total));
            }
            const uint64_t db = bits64(d);
            const uint64_t dm = db & 0x7fffffffffffffffull;
            const bool negative = (db >> 63) && dm;
            if (negative || (dm == 0 && rad_hi > 0.0f)) indefinite = 1;
            bool below;  // Q_ii < the FP64 column-order radius
            if (negative) {
                below = true;
            } else if (dm < widen_bits(__float_as_uint(rad_lo))) {
                below = true;
            } else if (dm >= widen_bits(__float_as_uint(rad_hi))) {
                below = false;
            } else {
                double radius = 0.0;
                for (int k = a; k < b; ++k)
                    if (__ldg(col + k) != r) radius += fabs(__ldg(val + k));
                below = d < radius;
            }
            if (below) nondominant = 1;
            if (offd) flags |= kGateOffDiagonal;
            if (negative || dm == 0 || dm > 0x7ff0000000000000ull) flags |= kGateNonPositive;  // !(Q_ii > 0)
            if (diag) diag[r] = d;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = umax64(best, shfl_xor(best, o));
    indefinite = __reduce_or_sync(0xffffffffu, indefinite);
    nondominant = __reduce_or_sync(0xffffffffu, nondominant);
    flags = static_cast<int>(__reduce_or_sync(0xffffffffu, static_cast<unsigned>(flags)));
    if (lane == 0) {
        if (best) atomicMax(&out->lip_bits, best);
        if (indefinite) atomicOr(&out->indefinite, 1);
        if (nondominant) atomicOr(&out->nondominant, 1);
        if (flags) atomicOr(&out->flags, flags);
    }
}

// Mixed engine, per row after the gate: 1/Q_ii (the polish's Jacobi preconditioner), the
// preconditioner scale v_r = Q_ii^-1/2 (rows without a positive diagonal L^-1/2), the FP32 cost
// and the FP32 bounds rounded inward (l32 = smallest float >= l, u32 = largest float <= u, so FP32
// iterates never leave the FP64 box).  Both scalings only precondition, so for 2^-100 <= Q_ii <
// 2^100 they come from the correctly rounded FP32 reciprocal and reciprocal square root of
// RN32(Q_ii) (two FP64 conversions per row instead of an FP64 division and square root); v is
// kept as that float in sstep (read by the bound of the scaled matrix, then overwritten by the
// steps) and widened exactly into s (free until the polish).
// The conversions run in integer arithmetic (rn_float*, ru_float, rd_float, widen_float: the same
// bits as the FP64 conversion instructions, which GB300 issues at 1/64 of the FP32 rate), and
// the rows outside the window take FP64 arithmetic alone.
__global__ void __launch_bounds__(kBlock) prepare_kernel(InstDev I, int n) {
    const int stride = gridDim.x * blockDim.x;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        const double d = I.diag[r];
        const uint64_t db = bits64(d);
        const int e = static_cast<int>(db >> 52);  // biased exponent; sign set => outside
        double dinv;
        float v;
        if (e >= 923 && e < 1123) {
            const float df = rn_float(d);
            dinv = widen_float(__frcp_rn(df));
            v = __frsqrt_rn(df);
        } else if (d > 0) {
            dinv = 1.0 / d;
            v = __double2float_rn(1.0 / sqrt(d));
        } else {
            dinv = 1.0;
            v = __double2float_rn(1.0 / sqrt(gate_lipschitz(I)));
        }
        const_cast<double*>(I.dinv)[r] = dinv;
        I.s[r] = widen_float(v);
        I.sstep[r] = v;
        const_cast<float*>(I.c32)[r] = rn_float_all(I.c[r]);
        const_cast<float*>(I.l32)[r] = ru_float(I.l[r]);
        const_cast<float*>(I.u32)[r] = rd_float(I.u[r]);
    }
}

// Diagonally preconditioned FISTA (mixed engine): FISTA on y = D^1/2 x (D = diag Q) is FISTA on
// x with the per-row step v_i^2 / L', v_i = Q_ii^-1/2 (rows without a positive diagonal keep
// v_i = L^-1/2, L the plain Gershgorin bound) and L' = max_i v_i sum_j |Q_ij| v_j, the Gershgorin
// bound of V Q V.  The box stays a box, so the projection maps over unchanged.  prepare_kernel
// leaves v (an FP32 value) in sstep and, widened, in the s array.

// L' as an upper bound in FP32 arithmetic rounded up: |Q_ij| <= |hi_ij| plus one unit (hi the
// nearest float), every product and sum rounded up, so the result is at least the exact bound
// of V Q V for the v the steps use (FP64 per nonzero would cost more than the pass's bytes).
template <int LANES>
__global__ void __launch_bounds__(kBlock) precond_bound_kernel(InstDev I, int n) {
    constexpr int R = 32 / LANES;
    const int lane = threadIdx.x & 31, sl = lane % LANES;
    const int groups = gridDim.x * (kBlock / 32) * R;
    const float* __restrict__ vf = I.sstep;
    uint32_t best = 0;
    for (int base = (blockIdx.x * (kBlock / 32) + (threadIdx.x >> 5)) * R; base < n; base += groups) {
        const int r = base + lane / LANES;
        float sum = 0.0f;
        if (r < n) {
            const int ks = __ldg(I.rowptr + r), ke = __ldg(I.rowptr + r + 1);
            for (int k = ks + sl; k < ke; k += LANES) {
                const uint32_t hb = __float_as_uint(__ldg(I.vhi + k)) & 0x7fffffffu;
                const float q = __uint_as_float(hb >= 0x7f800000u ? 0x7f800000u : hb + 1u);
                const int32_t c = __ldg(I.col + k);  // in range once the gate passes; clamped until then
                sum = __fmaf_ru(q, __ldg(vf + (static_cast<uint32_t>(c) < static_cast<uint32_t>(n) ? c : 0)), sum);
            }
        }
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) sum = __fadd_ru(sum, __shfl_xor_sync(0xffffffffu, sum, o));
        if (r < n && sl == 0) best = max(best, __float_as_uint(__fmul_ru(sum, vf[r])));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (best && best < 0x00800000u) best = 0x00800000u;  // a subnormal bound: 2^-126 above it
    if ((threadIdx.x & 31) == 0 && best)
        atomicMax(reinterpret_cast<unsigned long long*>(I.lprec), static_cast<unsigned long long>(widen_bits(best)));
}

// scaled = 0: the scalar step 1/L in every row (L from lprec under the power estimate); scaled:
// v^2 / L' rounded down in FP32 (v read from sstep before the step replaces it).
__global__ void __launch_bounds__(kBlock) precond_step_kernel(InstDev I, int n, int scaled) {
    const int stride = gridDim.x * blockDim.x;
    const double lp = (scaled || I.lip_device) ? *I.lprec : 0.0;
    const bool per_row = scaled && lp > 0;
    // per thread setup: the FP64 division of the scalar step only where it is used
    const float plain =
        per_row ? 0.0f : static_cast<float>((I.lip_device && lp > 0) ? 1.0 / lp : 1.0 / gate_lipschitz(I));
    const float inv = per_row ? __frcp_rd(ru_float(lp)) : 0.0f;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += stride) {
        float s = plain;
        if (per_row) {
            const float v = I.sstep[r];
            s = __fmul_rd(__fmul_rd(v, v), inv);
        }
        I.sstep[r] = s;
    }
}

// ---- power-iteration (Lanczos) Lipschitz estimate (BQP_LIPSCHITZ_POWER) ---------------------------
// Estimates lambda_max of M = S Q S (S = diag(v) for the preconditioned mixed engine, else the
// identity) in FP64 at admission.  The power iteration's Krylov space {y0, M y0, M^2 y0, ...}
// from a fixed positive pseudo-random y0 is spanned by the Lanczos process (the power iteration
// alone converges too slowly where the top eigenvalues cluster, as on graph Laplacians):
//     v_k = w_k / beta_k,  z = M v_k,  alpha_k = v_k'z,  w_k+1 = z - alpha_k v_k - beta_k v_k-1,
// kLanczosSteps steps, two kernels per step (product with alpha; update with beta).  The last
// block of the final update takes the largest eigenvalue theta of the tridiagonal T (Sturm
// bisection) and its residual |beta_K s_K| (s the unit eigenvector of T), and writes
//     L = min(Gershgorin bound of M, max(theta + residual, 1.001 theta))
// to lprec: theta <= lambda_max, and some eigenvalue of M lies within the residual of theta.
// An invariant subspace (beta ~ 0, e.g. n < kLanczosSteps) ends the process early.
// Deterministic: fixed grid, fixed shuffle trees, the last block adds the block partials in order.
constexpr int kLanczosSteps = 32;
constexpr int kLanczosBlocks = 152 * 4;
struct LanczosState {
    double alpha[kLanczosSteps];
    double beta[kLanczosSteps + 1];  // beta[0] = |y0|, beta[k + 1] = |w_k+1|
    unsigned ticket;
    int steps;                       // alpha's computed; the process stops early at a zero beta
    int stopped;
    int pad;
};

__device__ __forceinline__ double lanczos_start(int r) {
    return 0.5 + static_cast<double>(mix_index(static_cast<unsigned>(r) * 2654435761u + 12345u) >> 8) * (1.0 / 16777216.0);
}

// Block sum of one double in a fixed order; the last block (ticket) adds the block partials with
// all its threads (strided, then the same tree) and returns true in its thread 0 with the grid
// total in *total.
__device__ __forceinline__ double lanczos_block_sum(double x, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += shfl_xor(x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    double b = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kBlock / 32; ++w) b += red[w];
    return b;  // thread 0
}

__device__ bool lanczos_reduce(double x, double* partial, LanczosState* st, double* total) {
    __shared__ double red[kBlock / 32];
    __shared__ int last;
    const double b = lanczos_block_sum(x, red);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1 ? 1 : 0;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double t = 0;
    for (unsigned k = threadIdx.x; k < gridDim.x; k += kBlock) t += __ldcg(partial + k);
    t = lanczos_block_sum(t, red);  // thread 0 read red before the barrier above
    if (threadIdx.x != 0) return false;
    st->ticket = 0;
    *total = t;
    return true;
}

// w = y0, beta_0 = |y0|
__global__ void __launch_bounds__(kBlock) lanczos_init_kernel(int n, double* __restrict__ w, double* __restrict__ partial,
                                                              LanczosState* st) {
    double b = 0;
    for (int r = blockIdx.x * kBlock + threadIdx.x; r < n; r += gridDim.x * kBlock) {
        const double y = lanczos_start(r);
        w[r] = y;
        b += y * y;
    }
    double t;
    if (lanczos_reduce(b, partial, st, &t)) st->beta[0] = sqrt(t);
}

// step k: v_k = w / beta_k (stored), z = M v_k, alpha_k = v_k' z
__global__ void __launch_bounds__(kBlock) lanczos_product_kernel(InstDev I, int n, const double* __restrict__ val, int scaled,
                                                                 const double* __restrict__ w, double* __restrict__ vk,
                                                                 double* __restrict__ z, double* __restrict__ partial,
                                                                 LanczosState* st, int k) {
    if (st->stopped) return;
    const double scale = 1.0 / st->beta[k];
    const double* __restrict__ v = I.s;
    double a = 0;
    for (int r = blockIdx.x * kBlock + threadIdx.x; r < n; r += gridDim.x * kBlock) {
        const int ks = __ldg(I.rowptr + r), ke = __ldg(I.rowptr + r + 1);
        double acc = 0;
        for (int q = ks; q < ke; ++q) {
            int j = __ldg(I.col + q);
            if (static_cast<uint32_t>(j) >= static_cast<uint32_t>(n)) j = 0;  // until the gate has checked it
            acc += val[q] * (scaled ? v[j] * w[j] : w[j]);
        }
        if (scaled) acc *= v[r];
        const double zr = acc * scale, vr = w[r] * scale;
        z[r] = zr;
        vk[r] = vr;
        a += vr * zr;
    }
    double t;
    if (lanczos_reduce(a, partial, st, &t)) {
        st->alpha[k] = t;
        st->steps = k + 1;
    }
}

// Largest eigenvalue of the m x m tridiagonal (alpha, beta[1..m-1]) and the residual of its Ritz
// pair, |beta_m s_m| with s the unit eigenvector.  One thread.
__device__ void lanczos_ritz(const LanczosState* st, int m, double* theta_out, double* resid_out) {
    const double* a = st->alpha;
    const double* b = st->beta;  // off-diagonal i (between i-1 and i) is b[i], i = 1..m-1
    double lo = a[0], hi = a[0];
    for (int i = 0; i < m; ++i) {
        const double rad = (i > 0 ? fabs(b[i]) : 0.0) + (i + 1 < m ? fabs(b[i + 1]) : 0.0);
        lo = fmin(lo, a[i] - rad);
        hi = fmax(hi, a[i] + rad);
    }
    // Sturm count of eigenvalues > x: negative pivots of T - x I counted from the bottom
    for (int it = 0; it < 200 && hi - lo > 1e-15 * fmax(fabs(hi), fabs(lo)); ++it) {
        const double x = 0.5 * (lo + hi);
        int below = 0;
        double d = 1.0;
        for (int i = 0; i < m; ++i) {
            const double off = i > 0 ? b[i] * b[i] : 0.0;
            d = (a[i] - x) - (i > 0 ? off / (d != 0.0 ? d : 1e-300) : 0.0);
            if (d < 0) ++below;
        }
        if (below < m) lo = x;  // some eigenvalue lies above x
        else hi = x;
    }
    const double theta = hi;
    // eigenvector of T for theta by the three-term recurrence from s_0 = 1, kept normalised
    double s_prev = 0.0, s_cur = 1.0, norm2 = 1.0;
    for (int i = 0; i + 1 < m; ++i) {
        double s_next = ((theta - a[i]) * s_cur - (i > 0 ? b[i] * s_prev : 0.0)) / (b[i + 1] != 0.0 ? b[i + 1] : 1e-300);
        norm2 += s_next * s_next;
        s_prev = s_cur;
        s_cur = s_next;
        if (norm2 > 1e200) {
            const double f = 1.0 / sqrt(norm2);
            s_prev *= f;
            s_cur *= f;
            norm2 = 1.0;
        }
    }
    *theta_out = theta;
    *resid_out = fabs(b[m]) * fabs(s_cur) / sqrt(norm2);
}

// w_k+1 = z - alpha_k v_k - beta_k v_k-1, beta_k+1 = |w_k+1|; the final step writes the estimate
__global__ void __launch_bounds__(kBlock) lanczos_update_kernel(InstDev I, int n, const double* __restrict__ z,
                                                                const double* __restrict__ vk,
                                                                const double* __restrict__ vprev, double* __restrict__ w,
                                                                double* __restrict__ partial, LanczosState* st, int k) {
    if (st->stopped) return;
    const double al = st->alpha[k], be = k > 0 ? st->beta[k] : 0.0;
    double b = 0;
    for (int r = blockIdx.x * kBlock + threadIdx.x; r < n; r += gridDim.x * kBlock) {
        const double x = z[r] - al * vk[r] - (k > 0 ? be * vprev[r] : 0.0);
        w[r] = x;
        b += x * x;
    }
    double t;
    if (!lanczos_reduce(b, partial, st, &t)) return;
    const double beta = sqrt(t);
    st->beta[k + 1] = beta;
    const bool invariant = !(beta > 1e-12 * fmax(fabs(al), 1e-300));
    if (invariant) st->stopped = 1;
    if (invariant || k + 1 == kLanczosSteps) {
        if (invariant) st->beta[k + 1] = 0.0;
        double theta, resid;
        lanczos_ritz(st, k + 1, &theta, &resid);
        const double est = fmax(theta + resid, 1.001 * theta);
        if (isfinite(est) && est > 0) *I.lprec = fmin(*I.lprec, est);  // lprec: the Gershgorin bound of M
    }
}

// ---- standalone check on caller arrays ---------------------------------------------------------
struct StandaloneScratch {
    int done;
    int pad[3];
};

__global__ void __launch_bounds__(kBlock) check_standalone_kernel(CheckSrc s, int n, double tol, double offset,
                                                                 Partial* partial, StandaloneScratch* scr,
                                                                 double* result) {
    const int rows_per_block = (n + gridDim.x - 1) / gridDim.x;
    const int rb = blockIdx.x * rows_per_block;
    const int re = min(n, rb + rows_per_block);
    Acc a = acc_identity();
    if (rb < re) check_rows<0>(s, VAR_WARP, rb, re, a);
    Acc total = block_reduce(a);
    __shared__ int is_last;
    if (threadIdx.x == 0) {
        store_partial(&partial[blockIdx.x], total);
        __threadfence();
        is_last = atomicAdd(&scr->done, 1) == static_cast<int>(gridDim.x) - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    Acc acc = acc_identity();
    for (int k = threadIdx.x; k < static_cast<int>(gridDim.x); k += kBlock) acc = combine(acc, load_partial(&partial[k]));
    Acc tot = block_reduce(acc);
    if (threadIdx.x == 0) {
        scr->done = 0;
        double obj, stat, prim, bound, gap;
        if (tot.flags & 1) {
            obj = __longlong_as_double(0x7ff8000000000000LL);
            stat = kInf; prim = kInf; bound = -kInf; gap = kInf;
        } else {
            obj = tot.obj + offset;
            stat = bdouble(tot.stat);
            prim = bdouble(tot.prim);
            if (s.gate) bound = tot.sep + offset;
            else bound = (tot.flags & 2) ? -kInf : obj + tot.bnd;
            gap = isfinite(bound) ? fabs(obj - bound) / (1.0 + fabs(obj)) : kInf;
        }
        bool verified = isfinite(obj) && smax(prim, smax(stat, 0.0)) <= tol;
        if (s.gate) verified = verified && gap <= tol;
        result[0] = obj;
        result[1] = prim;
        result[2] = stat;
        result[3] = 0.0;
        result[4] = bound;
        result[5] = gap;
        result[6] = verified ? 1.0 : 0.0;
        result[7] = static_cast<double>(tot.nact);
    }
}

// ---- plugin-level FISTA step --------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) box_step_kernel(int n, const int32_t* __restrict__ rowptr,
                                                          const int32_t* __restrict__ col,
                                                          const double* __restrict__ val,
                                                          const double* __restrict__ c,
                                                          const double* __restrict__ l,
                                                          const double* __restrict__ u, double L, double beta,
                                                          double* __restrict__ x, const double* __restrict__ w_in,
                                                          double* __restrict__ w_out) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double acc = 0.0;
        const int ks = __ldg(rowptr + r), ke = __ldg(rowptr + r + 1);
        for (int k = ks; k < ke; ++k) acc = __dadd_rn(acc, __dmul_rn(__ldg(val + k), __ldg(w_in + __ldg(col + k))));
        const double v = __dsub_rn(__ldg(w_in + r), __ddiv_rn(__dadd_rn(acc, __ldg(c + r)), L));
        const double nx = smax(__ldg(l + r), smin(__ldg(u + r), v));
        w_out[r] = __dadd_rn(nx, __dmul_rn(beta, __dsub_rn(nx, x[r])));
        x[r] = nx;
    }
}

}  // namespace

// ---- launch wrappers -----------------------------------------------------------------------------
namespace {
// One full wave (SMs x resident blocks per SM) per tile kernel, computed once per process.
struct Waves {
    int group[kStepGroups] = {};
    int exact = 0;
    int check = 0, check_mixed = 0, check_verify = 0, polish = 0, matvec = 0, residual = 0;
};
Waves g_waves;

template <class K>
int wave_of(K kernel, int sms, int dyn_smem) {
    if (dyn_smem > 0) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_smem);
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kBlock, dyn_smem);
    return sms * (b < 1 ? 1 : b);
}
constexpr int kSmemF32 = smem_bytes<float>() > kTileNnz * 4 ? smem_bytes<float>() : kTileNnz * 4;
constexpr int kSmem8 = smem_bytes<double>() > kTileNnz * 8 ? smem_bytes<double>() : kTileNnz * 8;
inline int pick(int cap, int wave) { return cap < wave ? (cap < 1 ? 1 : cap) : wave; }

// Dynamic shared memory of a step group: the block- and warp-staged structures keep their
// products there, the sub-warp ones none.
template <int PREC, int VAR>
constexpr int step_smem() {
    return (VAR == VAR_TILE || VAR == VAR_WARP) ? (PREC == PREC_MIXED ? kSmemF32 : kSmem8) : 0;
}

template <int PREC, int VAR>
void group_wave(int sms) {
    g_waves.group[step_group(PREC, VAR)] = wave_of(step_kernel<PREC, VAR>, sms, step_smem<PREC, VAR>());
}

template <int PREC>
void group_waves(int sms) {
    group_wave<PREC, VAR_TILE>(sms);
    group_wave<PREC, 1>(sms);
    group_wave<PREC, 2>(sms);
    group_wave<PREC, 4>(sms);
    group_wave<PREC, 8>(sms);
    group_wave<PREC, 16>(sms);
    group_wave<PREC, 32>(sms);
    group_wave<PREC, VAR_WARP>(sms);
}

template <int PREC, int VAR>
void launch_group(const View& v, int group, int j, int grid, cudaStream_t s) {
    step_kernel<PREC, VAR><<<pick(grid, g_waves.group[group]), kBlock, step_smem<PREC, VAR>(), s>>>(v, group, j);
}

template <int PREC>
void launch_group_of(const View& v, int group, int j, int grid, cudaStream_t s) {
    switch (group % kVariants) {
    case 0: launch_group<PREC, VAR_TILE>(v, group, j, grid, s); break;
    case 1: launch_group<PREC, 1>(v, group, j, grid, s); break;
    case 2: launch_group<PREC, 2>(v, group, j, grid, s); break;
    case 3: launch_group<PREC, 4>(v, group, j, grid, s); break;
    case 4: launch_group<PREC, 8>(v, group, j, grid, s); break;
    case 5: launch_group<PREC, 16>(v, group, j, grid, s); break;
    case 6: launch_group<PREC, 32>(v, group, j, grid, s); break;
    default: launch_group<PREC, VAR_WARP>(v, group, j, grid, s); break;
    }
}
}  // namespace

int tile_grid(int sms) {
    group_waves<PREC_FP64>(sms);
    group_waves<PREC_MIXED>(sms);
    g_waves.exact = wave_of(step_exact_kernel, sms, 0);
    g_waves.check = wave_of(check_kernel<FAMILY_FP64>, sms, kSmem8);
    g_waves.check_mixed = wave_of(check_kernel<FAMILY_MIXED>, sms, kSmem8);
    g_waves.check_verify = wave_of(check_kernel<FAMILY_VERIFY>, sms, kSmem8);
    g_waves.matvec = wave_of(cg_matvec_kernel, sms, 0);
    g_waves.residual = wave_of(polish_residual_kernel, sms, 0);
    wave_of(check_standalone_kernel, sms, kSmem8);
    g_waves.polish = wave_of(cg_vector_kernel, sms, 0);
    int m = g_waves.exact;
    for (int w : g_waves.group) m = w > m ? w : m;
    for (int w : {g_waves.check, g_waves.matvec, g_waves.polish})
        m = w > m ? w : m;
    return m;
}

int cg_matvec_slots() { return g_waves.matvec; }

void launch_check(const View& v, int grid, cudaStream_t s) {
    check_kernel<FAMILY_MIXED><<<pick(grid, g_waves.check_mixed), kBlock, kSmem8, s>>>(v);
    check_kernel<FAMILY_VERIFY><<<pick(grid, g_waves.check_verify), kBlock, kSmem8, s>>>(v);
    check_kernel<FAMILY_FP64><<<pick(grid, g_waves.check), kBlock, kSmem8, s>>>(v);
}

void launch_step_group(const View& v, int group, int j, int grid, cudaStream_t s) {
    if (group >= kVariants) launch_group_of<PREC_MIXED>(v, group, j, grid, s);
    else launch_group_of<PREC_FP64>(v, group, j, grid, s);
}

void launch_step_exact(const View& v, int j, int grid, cudaStream_t s) {
    step_exact_kernel<<<pick(grid, g_waves.exact), kBlock, 0, s>>>(v, j);
}

void launch_polish_init(const View& v, int grid, cudaStream_t s) {
    polish_init_kernel<<<pick(grid, g_waves.polish), kBlock, 0, s>>>(v);
}
void launch_polish_residual(const View& v, int grid, cudaStream_t s) {
    polish_residual_kernel<<<pick(grid, g_waves.residual), kBlock, 0, s>>>(v);
}
void launch_cg_matvec(const View& v, int grid, cudaStream_t s) {
    cg_matvec_kernel<<<pick(grid, g_waves.matvec), kBlock, 0, s>>>(v);
}
void launch_cg_vector(const View& v, int grid, cudaStream_t s, cudaGraphConditionalHandle cg_loop, int cap) {
    cg_vector_kernel<<<pick(grid, g_waves.polish), kBlock, 0, s>>>(v, cg_loop, cap);
}

void launch_gate(const View& v, const cudaGraphConditionalHandle* fista, cudaGraphConditionalHandle polish,
                 cudaGraphConditionalHandle cg_loop, StepLaunches steps, int body_steps, cudaStream_t s) {
    gate_kernel<<<1, 1024, 0, s>>>(v, fista[0], fista[1], fista[2], polish, cg_loop, steps, body_steps);
}
void launch_control(const View& v, cudaGraphConditionalHandle loop, int steps, cudaStream_t s) {
    control_kernel<<<1, 1024, 0, s>>>(v, loop, steps);
}
void launch_gate_plain(const View& v, int steps, cudaStream_t s) { gate_plain_kernel<<<1, 1024, 0, s>>>(v, steps); }
void launch_control_plain(const View& v, int steps, cudaStream_t s) { control_plain_kernel<<<1, 1024, 0, s>>>(v, steps); }

void launch_init_instance(const View& v, int slot, int n, int precision, cudaStream_t s) {
    int grid = (n + kBlock - 1) / kBlock;
    if (grid > 4096) grid = 4096;
    if (grid < 1) grid = 1;
    (void)precision;
    init_instance_kernel<<<grid, kBlock, 0, s>>>(v, slot, n);
}

void launch_rearm(const View& v, const InstDev* stage, const int32_t* slots, const int2* spans, int n_spans,
                  cudaStream_t s) {
    if (n_spans > 0) rearm_kernel<<<n_spans, kBlock, 0, s>>>(v, stage, slots, spans);
}

// Lanes per row of the admission kernels: the residual pass's choice (about a sixth of the
// average row length), clamped to 2..8.
inline int row_lanes(const InstDev& rec) { return rec.lanes_res >= 8 ? 8 : rec.lanes_res >= 4 ? 4 : 2; }

void launch_precondition(const InstDev& rec, int64_t n, const double* val, bool scaled, void* power_scratch,
                         cudaStream_t s) {
    int64_t grid = (n + kBlock - 1) / kBlock;
    if (grid > 152 * 16) grid = 152 * 16;
    if (grid < 1) grid = 1;
    if (scaled) {
        cudaMemsetAsync(rec.lprec, 0, sizeof(double), s);
        const int lanes = row_lanes(rec);
        int64_t g = (n * lanes + kBlock - 1) / kBlock;
        if (g > 152 * 16) g = 152 * 16;
        if (g < 1) g = 1;
        const int gi = static_cast<int>(g), ni = static_cast<int>(n);
        if (lanes == 8) precond_bound_kernel<8><<<gi, kBlock, 0, s>>>(rec, ni);
        else if (lanes == 4) precond_bound_kernel<4><<<gi, kBlock, 0, s>>>(rec, ni);
        else precond_bound_kernel<2><<<gi, kBlock, 0, s>>>(rec, ni);
    }
    if (rec.lip_device) {
        if (!scaled) cudaMemcpyAsync(rec.lprec, &rec.gate->lip_bits, sizeof(double), cudaMemcpyDeviceToDevice, s);
        launch_power_lipschitz(rec, n, val, scaled, power_scratch, s);
    }
    precond_step_kernel<<<static_cast<int>(grid), kBlock, 0, s>>>(rec, static_cast<int>(n), scaled ? 1 : 0);
}

inline size_t round256(size_t b) { return (b + 255) / 256 * 256; }

size_t power_scratch_bytes(int64_t n) {
    return 1024 + round256(sizeof(double) * kLanczosBlocks) + 4 * round256(sizeof(double) * static_cast<size_t>(n));
}

void launch_power_lipschitz(const InstDev& rec, int64_t n, const double* val, bool scaled, void* scratch, cudaStream_t s) {
    char* base = static_cast<char*>(scratch);
    LanczosState* st = reinterpret_cast<LanczosState*>(base);
    static_assert(sizeof(LanczosState) <= 1024, "state size");
    double* partial = reinterpret_cast<double*>(base + 1024);
    const size_t vec = round256(sizeof(double) * static_cast<size_t>(n));
    char* vecs = base + 1024 + round256(sizeof(double) * kLanczosBlocks);
    double* w = reinterpret_cast<double*>(vecs);
    double* z = reinterpret_cast<double*>(vecs + vec);
    double* va = reinterpret_cast<double*>(vecs + 2 * vec);
    double* vb = reinterpret_cast<double*>(vecs + 3 * vec);
    cudaMemsetAsync(st, 0, sizeof(LanczosState), s);
    int64_t g = (n + kBlock - 1) / kBlock;
    if (g > kLanczosBlocks) g = kLanczosBlocks;
    if (g < 1) g = 1;
    const int grid = static_cast<int>(g), ni = static_cast<int>(n);
    lanczos_init_kernel<<<grid, kBlock, 0, s>>>(ni, w, partial, st);
    for (int k = 0; k < kLanczosSteps; ++k) {
        double* vk = (k & 1) ? vb : va;
        double* vprev = (k & 1) ? va : vb;
        lanczos_product_kernel<<<grid, kBlock, 0, s>>>(rec, ni, val, scaled ? 1 : 0, w, vk, z, partial, st, k);
        lanczos_update_kernel<<<grid, kBlock, 0, s>>>(rec, ni, z, vk, vprev, w, partial, st, k);
    }
}

void launch_gate_raw(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val, GateResult* out,
                     double* diag, float* vhi, float* vlo, cudaStream_t s) {
    cudaMemsetAsync(out, 0, sizeof(GateResult), s);
    const int64_t groups = (n + 31) / 32;
    int64_t grid = (groups + kGateWarps - 1) / kGateWarps;
    if (grid > 152 * 8) grid = 152 * 8;
    if (grid < 1) grid = 1;
    convexity_gate_kernel<<<static_cast<int>(grid), kGateWarps * 32, 0, s>>>(rowptr, col, val, static_cast<int>(n), out,
                                                                             diag, vhi, vlo);
}

void launch_gate(const InstDev& rec, int64_t n, const double* val, cudaStream_t s) {
    const bool split = rec.precision == PREC_MIXED;
    launch_gate_raw(n, rec.rowptr, rec.col, val, rec.gate, const_cast<double*>(rec.diag),
                    split ? const_cast<float*>(rec.vhi) : nullptr, split ? const_cast<float*>(rec.vlo) : nullptr, s);
}

void launch_prepare_instance(const InstDev& rec, int64_t n, cudaStream_t s) {
    if (rec.precision != PREC_MIXED) return;  // the gate already stored the FP64 engine's diagonal
    int64_t grid = (n + kBlock - 1) / kBlock;
    if (grid > 152 * 16) grid = 152 * 16;
    if (grid < 1) grid = 1;
    prepare_kernel<<<static_cast<int>(grid), kBlock, 0, s>>>(rec, static_cast<int>(n));
}

int check_grid(int64_t n) {
    int64_t g = (n + 4095) / 4096;
    if (g > 2048) g = 2048;
    if (g < 1) g = 1;
    return static_cast<int>(g);
}

size_t check_scratch_bytes(int64_t n) {
    return sizeof(Partial) * static_cast<size_t>(check_grid(n)) + 256;
}

void launch_check_standalone(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                             const double* x, const double* c, const double* l, const double* u,
                             double tol, double offset, int gate, void* scratch, double* result,
                             cudaStream_t s) {
    CheckSrc src{};
    src.rowptr = rowptr; src.col = col; src.val64 = val; src.x64 = x; src.c = c; src.l = l; src.u = u;
    src.diag = nullptr;  // a diagonal Hessian's only entry per row is its diagonal
    src.gate = gate;
    const int grid = check_grid(n);
    // The kernel's dynamic shared memory plus its static reduction buffer exceed the default
    // 48 KB: opt in on every call (a cheap host call; a per-device flag would go stale when the
    // caller resets the device and its context is recreated).
    cudaFuncSetAttribute(check_standalone_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem8);
    auto* scr = static_cast<StandaloneScratch*>(scratch);
    auto* partial = reinterpret_cast<Partial*>(static_cast<char*>(scratch) + 256);
    check_standalone_kernel<<<grid, kBlock, kSmem8, s>>>(src, static_cast<int>(n), tol, offset, partial, scr, result);
}

cudaError_t load_check_standalone() {
    cudaError_t e = cudaFuncSetAttribute(check_standalone_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem8);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes attr;
    return cudaFuncGetAttributes(&attr, check_standalone_kernel);
}

void launch_box_step(int64_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                     const double* c, const double* l, const double* u, double L, double beta,
                     double* x, const double* w_in, double* w_out, cudaStream_t s) {
    int grid = static_cast<int>((n + kBlock - 1) / kBlock);
    if (grid > 152 * 16) grid = 152 * 16;
    if (grid < 1) grid = 1;
    box_step_kernel<<<grid, kBlock, 0, s>>>(static_cast<int>(n), rowptr, col, val, c, l, u, L, beta, x, w_in, w_out);
}

}  // namespace bqp
