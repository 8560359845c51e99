// batch.cu -- the batching form: thousands of small circuits in one
// persistent launch, replayed from a CUDA graph.
//
// Each instance is a hardware-efficient ansatz on n qubits: L layers of
// rotateY on every qubit, rotateZ on every qubit, then controlNot(q, q+1)
// for q = 0..n-2; afterwards prob(q, 0) and prob(q, 1) for every q and a
// sampleAll draw per uniform.  The per-instance result is the one qsl's
// Default backend gives for the same calls (gates.cpp, measure.cpp), bit
// for bit: every amplitude sees the reference's operations in the
// reference's order with its rounding, the probabilities are sequential
// sums in index order, and the sampling CDF is the sequential double sum
// merged against the instance's sorted uniforms (the first index whose
// running sum reaches a uniform is its outcome, as drawSample's search
// returns, measure.cpp:164-188).
//
// The CDF is one running sum per instance, a chain of dependent FP64 adds,
// and the FP64 pipe takes as long for one active lane as for 32.  So
// k_batch leaves each instance's |a|^2 terms in global memory and a second
// kernel in the same graph, k_batch_cdf, walks the CDFs one instance per
// thread: each FP64 instruction then advances up to 32 of them.
//
// Schedule: persistent CTAs pull instances, largest first, from an atomic
// counter.  A state of at most one tile (2^k amplitudes of shared memory)
// lives in shared memory for its whole circuit.  A larger state lives in
// two buffers of the CTA's slot in a global arena and takes two passes per
// layer instead of one per gate:
//   pass 1  tiles of 2^k consecutive amplitudes: rotateY on qubits 0..k-1;
//   pass 2  tiles that vary the high n-k qubits and the lowest 2k-n ones:
//           rotateY on qubits k..n-1, then rotateZ on every qubit (each
//           rotateZ touches one amplitude at a time, so all n of them apply
//           per amplitude, in order), then the whole controlNot ladder as
//           one permutation into the other buffer.
// The ladder maps basis index x to y with y_i = x_0 ^ ... ^ x_i (each
// controlNot(q, q+1) flips bit q+1 when bit q of the running index is set);
// a pass-2 tile writes its outputs in runs of consecutive y.
//
// The tile size, threads per CTA and CTAs per SM are picked by measuring
// the candidates on the caller's own batch (qslc_batch_autotune).
#include "gatemath.cuh"
#include "replay.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>
#include <vector>

namespace qslc {
namespace {

constexpr int MAX_Q = 26;
constexpr int CDF_THREADS = 128;   // 4 warps, 4 instances
// How the rotation outputs are computed (complex128), as mode masks
// (gatemath.cuh, OutMode): rotateY cycles over a thread's successive pairs
// through three 8-bit masks, rotateZ over the qubits through three (2 bits
// per output).  The build can set others (-DQSLC_BATCH_MODES_RY=...,
// -DQSLC_BATCH_MODES_RZ=...) for tuning.
#ifndef QSLC_BATCH_MODES_RY
#define QSLC_BATCH_MODES_RY 0x555555u
#endif
#ifndef QSLC_BATCH_MODES_RZ
#define QSLC_BATCH_MODES_RZ 0x050505u
#endif
constexpr unsigned BATCH_MODES_RY = QSLC_BATCH_MODES_RY;
constexpr unsigned BATCH_MODES_RZ = QSLC_BATCH_MODES_RZ;

struct InstDesc {
    uint32_t n, L;
    uint64_t coef;      // offset of its coefficients: L*n*4 values (cy, sy, cz, sz)
    uint64_t probs;     // offset of its 2n probabilities
    uint64_t shots;     // offset of its shots (sorted-uniform order)
    uint64_t norms;     // offset of its 2^n |a|^2 terms (doubles) for the sampling CDF
};

struct BatchArgs {
    const InstDesc *inst;
    const uint32_t *order;
    uint32_t ninst;
    unsigned *counter;
    const void *coef;
    void *probs;
    const double *usorted;
    uint64_t *shots;
    uint32_t nshots;
    double *norms;              // every instance's |a|^2 terms, in index order
    const uint32_t *cdf_order;  // instances by qubit count, largest first
    void *arena;
    uint64_t slot_amps;     // amplitudes per arena buffer (two buffers per slot)
    unsigned tile_log2;     // k: the shared-memory tile holds 2^k amplitudes
};

__host__ __device__ __forceinline__ uint64_t ladder(uint64_t x)
{   // y_i = x_0 ^ ... ^ x_i
    x ^= x << 1;
    x ^= x << 2;
    x ^= x << 4;
    x ^= x << 8;
    x ^= x << 16;
    return x;
}

// The coefficients of one layer, decoded for the integer path once per CTA.
template <class T>
struct LayerCoefs {
    Coef<T> ry[MAX_Q], rz[MAX_Q];
};

template <class T>
__device__ __forceinline__ Coef<T> dev_coef(T c, T s)
{
    Coef<T> k{};
    k.c = c;
    k.s = s;
    k.kc = emu::make_const(double(c));
    k.ks = emu::make_const(double(s));
    k.mc = emu::make_mulk(double(c));
    k.ms = emu::make_mulk(double(s));
    return k;
}

template <class T>
__device__ __forceinline__ void stage_layer(LayerCoefs<T> &lc, const T *cf, uint32_t n)
{
    const unsigned tid = threadIdx.x;
    if (tid < n) {
        lc.ry[tid] = dev_coef<T>(cf[4 * tid], cf[4 * tid + 1]);
        lc.rz[tid] = dev_coef<T>(cf[4 * tid + 2], cf[4 * tid + 3]);
    }
    __syncthreads();
}

// rotateY on qubit `bit` of a state or tile held at `st` (2^m amplitudes),
// gates.cpp:169-174; every thread's pairs cycle through BATCH_MODES_RY.
template <class T>
__device__ __forceinline__ void ry_sweep(cplx<T> *st, unsigned m, unsigned bit, const Coef<T> &k)
{
    const uint64_t half = uint64_t(1) << (m - 1), b = uint64_t(1) << bit;
    unsigned it = 0;
    for (uint64_t j = threadIdx.x; j < half; j += blockDim.x, it = (it == 2 ? 0 : it + 1)) {
        const uint64_t i0 = insert0(j, bit);
        cplx<T> a0 = st[i0], a1 = st[i0 | b];
        pair_update<T, P_RY>(a0, a1, k, (BATCH_MODES_RY >> (8 * it)) & 0xFFu);
        st[i0] = a0;
        st[i0 | b] = a1;
    }
}

// rotateY on qubit `b0` and then on qubit `b1` (b0 < b1) of a state or tile
// at `st`, in one sweep: each thread holds the four amplitudes that differ
// only in those two bits, applies the first gate to its two pairs and then
// the second gate to its two pairs.  Every amplitude sees the operations of
// the two sweeps in their order, so the bits are those of two ry_sweep
// calls, with one barrier instead of two.
template <class T>
__device__ __forceinline__ void ry_sweep2(cplx<T> *st, unsigned m, unsigned b0, unsigned b1, const Coef<T> &k0,
                                          const Coef<T> &k1)
{
    const uint64_t quarter = uint64_t(1) << (m - 2);
    const uint64_t B0 = uint64_t(1) << b0, B1 = uint64_t(1) << b1;
    for (uint64_t j = threadIdx.x; j < quarter; j += blockDim.x) {
        const uint64_t x = insert00(j, b0, b1);
        cplx<T> a00 = st[x], a01 = st[x | B0], a10 = st[x | B1], a11 = st[x | B0 | B1];
        pair_update<T, P_RY>(a00, a01, k0, BATCH_MODES_RY & 0xFFu);
        pair_update<T, P_RY>(a10, a11, k0, (BATCH_MODES_RY >> 8) & 0xFFu);
        pair_update<T, P_RY>(a00, a10, k1, (BATCH_MODES_RY >> 16) & 0xFFu);
        pair_update<T, P_RY>(a01, a11, k1, BATCH_MODES_RY & 0xFFu);
        st[x] = a00;
        st[x | B0] = a01;
        st[x | B1] = a10;
        st[x | B0 | B1] = a11;
    }
}

// rotateY on the qubits lo..hi-1 of the circuit, in order, on bits
// off + (q - lo) of a state or tile of 2^m amplitudes: two gates per sweep
// (ry_sweep2), the last one alone when their number is odd; a barrier after
// each sweep.
#ifndef QSLC_BATCH_RY_PAIRS
#define QSLC_BATCH_RY_PAIRS 1
#endif
template <class T>
__device__ __forceinline__ void ry_layer(cplx<T> *st, unsigned m, unsigned lo, unsigned hi, unsigned off,
                                         const LayerCoefs<T> &lc)
{
    unsigned q = lo;
    for (; QSLC_BATCH_RY_PAIRS && q + 1 < hi; q += 2) {
        ry_sweep2<T>(st, m, off + (q - lo), off + (q + 1 - lo), lc.ry[q], lc.ry[q + 1]);
        __syncthreads();
    }
    for (; q < hi; q++) {
        ry_sweep<T>(st, m, off + (q - lo), lc.ry[q]);
        __syncthreads();
    }
}

// rotateZ on qubits 0..n-1, in that order, of the amplitude at basis index
// x (gates.cpp:200-205): the |0> member takes (re*c + im*s, im*c - re*s),
// the |1> member (re*c - im*s, im*c + re*s).  Both are re*c + im*sg and
// im*c + re*(-sg) with sg = +-s, and RN(u*(-v)) = -RN(u*v), so one form
// serves both members without a branch on the bit.
template <class T>
__device__ __forceinline__ cplx<T> rz_all(cplx<T> a, uint64_t x, uint32_t n, const LayerCoefs<T> &lc)
{
    for (uint32_t q = 0; q < n; q++) {
        const Coef<T> &k = lc.rz[q];
        const bool one = (x >> q) & 1;
        const T sg = one ? -k.s : k.s;
        emu::MulConst ksg = k.ks, kneg = k.ks;
        emu::MulK msg = k.ms, mneg = k.ms;
        if (one) {
            ksg.sign ^= emu::SIGN;
            msg.sign ^= 0x80000000u;
        } else {
            kneg.sign ^= emu::SIGN;
            mneg.sign ^= 0x80000000u;
        }
        const unsigned md = (BATCH_MODES_RZ >> (8 * (q % 3))) & 0xFFu;
        const T re = a.x, im = a.y;
        a.x = dot2m<T, false>(mode_of(md, 0), re, k.c, k.kc, k.mc, im, sg, ksg, msg);
        a.y = dot2m<T, false>(mode_of(md, 1), im, k.c, k.kc, k.mc, re, -sg, kneg, mneg);
    }
    return a;
}

// The sampling CDF's test u <= run, for u in [0, 1) and run >= 0: the bit
// patterns of non-negative doubles order like their values, so integer
// compares keep it off the FP64 pipe.
__device__ __forceinline__ bool cdf_reached(double u, double run)
{
    return __double_as_longlong(u) <= __double_as_longlong(run);
}

// The measurements of one instance from its final state `st` in shared
// memory (natural order): its 2n probabilities, and its |a|^2 terms for the
// sampling CDF written to `gn` (as doubles).  `nrm`, when not null, is room
// for 2^n values of T: every thread then computes the terms once, in
// parallel, and the probability sums read them instead of recomputing them.
template <class T>
__device__ void finish_instance(const cplx<T> *st, T *nrm, const InstDesc &d, T *__restrict__ probs,
                                double *__restrict__ gn)
{
    const uint32_t n = d.n;
    const uint64_t dim = uint64_t(1) << n, half = dim >> 1;
    const unsigned tid = threadIdx.x;
    __syncthreads();                                  // the state's last writes
    for (uint64_t i = tid; i < dim; i += blockDim.x) {
        const T t = norm2_rn(st[i].x, st[i].y);
        if (nrm) nrm[i] = t;
        gn[i] = double(t);
    }
    if (nrm) __syncthreads();
    auto term = [&](uint64_t i) {
        if (nrm) return nrm[i];
        const cplx<T> a = st[i];
        return norm2_rn(a.x, a.y);
    };
    // prob(q, o): sequential Fp sums in index order (measure.cpp:126-147)
    if (tid < 2 * n) {
        const uint32_t q = tid >> 1, o = tid & 1;
        const uint64_t ob = uint64_t(o) << q;
        T p = T(0);
        for (uint64_t j = 0; j < half; j++) p = rn<T>::add(p, term(insert0(j, q) | ob));
        probs[d.probs + 2 * q + o] = p;
    }
    __syncthreads();
}

// The measurements of a large instance: the final state passes one tile at
// a time; all threads turn a tile into its |a|^2 terms, in shared memory for
// the probability sums and in `gn` for the sampling CDF, and every sum walks
// its terms of the tile in index order, so each keeps the reference's
// sequential order while reading each term once from global memory.
template <class T>
__device__ void finish_big(const cplx<T> *st, cplx<T> *sm, unsigned k, const InstDesc &d,
                           T *__restrict__ probs, double *__restrict__ gn)
{
    const uint32_t n = d.n;
    const uint64_t dim = uint64_t(1) << n, chunk = uint64_t(1) << k;
    const unsigned tid = threadIdx.x, nt = blockDim.x;
    const uint32_t q = tid >> 1, o = tid & 1;
    T *nrm = reinterpret_cast<T *>(sm);
    T p = T(0);
    for (uint64_t c = 0; c < (dim >> k); c++) {
        __syncthreads();
        for (uint64_t i = tid; i < chunk; i += nt) {
            const cplx<T> a = st[(c << k) + i];
            const T t = norm2_rn(a.x, a.y);
            nrm[i] = t;
            gn[(c << k) + i] = double(t);
        }
        __syncthreads();
        if (tid < 2 * n) {
            // prob(q, o): the terms with bit q == o (measure.cpp:126-147)
            if (q < k) {
                const uint64_t ob = uint64_t(o) << q;
                for (uint64_t j = 0; j < (chunk >> 1); j++) p = rn<T>::add(p, nrm[insert0(j, q) | ob]);
            } else if (((c >> (q - k)) & 1) == o) {
                for (uint64_t i = 0; i < chunk; i++) p = rn<T>::add(p, nrm[i]);
            }
        }
    }
    if (tid < 2 * n) probs[d.probs + 2 * q + o] = p;
    __syncthreads();
}

// An instance that fits one tile: the whole circuit in shared memory.
template <class T>
__device__ void run_small(cplx<T> *sm, LayerCoefs<T> &lc, const InstDesc &d, const T *coef)
{
    const uint32_t n = d.n;
    const uint64_t dim = uint64_t(1) << n;
    const unsigned tid = threadIdx.x, nt = blockDim.x;
    for (uint64_t i = tid; i < dim; i += nt) {
        cplx<T> z;
        z.x = T(i == 0 ? 1 : 0);
        z.y = T(0);
        sm[i] = z;
    }
    for (uint32_t l = 0; l < d.L; l++) {
        stage_layer<T>(lc, coef + d.coef + uint64_t(l) * n * 4, n);   // also orders the fill
        ry_layer<T>(sm, n, 0, n, 0, lc);
        for (uint64_t i = tid; i < dim; i += nt) sm[i] = rz_all<T>(sm[i], i, n, lc);
        __syncthreads();
        for (uint32_t q = 0; q + 1 < n; q++) {       // controlNot(q, q+1), gates.cpp:215-240
            const uint64_t cb = uint64_t(1) << q, tb = uint64_t(1) << (q + 1);
            for (uint64_t j = tid; j < (dim >> 2); j += nt) {
                const uint64_t x1 = insert00(j, q, q + 1) | cb;
                const cplx<T> a = sm[x1], b = sm[x1 | tb];
                sm[x1] = b;
                sm[x1 | tb] = a;
            }
            __syncthreads();
        }
    }
}

// An instance larger than a tile: two buffers in the CTA's arena slot, two
// passes per layer.  Returns the buffer that holds the final state.
template <class T>
__device__ cplx<T> *run_big(cplx<T> *sm, LayerCoefs<T> &lc, const InstDesc &d, const T *coef,
                            cplx<T> *buf0, cplx<T> *buf1, unsigned k)
{
    const uint32_t n = d.n;
    const uint64_t dim = uint64_t(1) << n, tile = uint64_t(1) << k;
    const unsigned tid = threadIdx.x, nt = blockDim.x;
    const unsigned h = n - k;                 // qubits above the tile (h <= k)
    const unsigned c = k - h;                 // low qubits that pass-2 tiles keep whole
    const uint64_t cmask = (uint64_t(1) << c) - 1;
    cplx<T> *src = buf0, *dst = buf1;
    for (uint64_t i = tid; i < dim; i += nt) {
        cplx<T> z;
        z.x = T(i == 0 ? 1 : 0);
        z.y = T(0);
        src[i] = z;
    }
    for (uint32_t l = 0; l < d.L; l++) {
        stage_layer<T>(lc, coef + d.coef + uint64_t(l) * n * 4, n);   // also orders the writes above
        // pass 1: rotateY on qubits 0..k-1, tile by tile, in place
        for (uint64_t t = 0; t < (dim >> k); t++) {
            cplx<T> *g = src + (t << k);
            for (uint64_t i = tid; i < tile; i += nt) sm[i] = g[i];
            __syncthreads();
            ry_layer<T>(sm, k, 0, k, 0, lc);
            for (uint64_t i = tid; i < tile; i += nt) g[i] = sm[i];
            __syncthreads();
        }
        // pass 2: tile t fixes bits c..k-1 of the index to t; local index
        // l = (high bits << c) | (low c bits)
        for (uint64_t t = 0; t < (uint64_t(1) << h); t++) {
            const uint64_t mid = t << c;
            for (uint64_t i = tid; i < tile; i += nt) sm[i] = src[((i >> c) << k) | mid | (i & cmask)];
            __syncthreads();
            ry_layer<T>(sm, k, k, n, c, lc);
            // outputs in order of their destination: o = (high bits << c) |
            // (low c bits of y); the source's low bits are the inverse of the
            // ladder on those c bits, so consecutive o land on consecutive y
            for (uint64_t o = tid; o < tile; o += nt) {
                const uint64_t ylow = o & cmask;
                const uint64_t xlow = (ylow ^ (ylow << 1)) & cmask;
                const uint64_t lidx = (o & ~cmask) | xlow;
                const uint64_t x = ((o >> c) << k) | mid | xlow;
                dst[ladder(x) & (dim - 1)] = rz_all<T>(sm[lidx], x, n, lc);
            }
            __syncthreads();
        }
        cplx<T> *tmp = src;
        src = dst;
        dst = tmp;
    }
    return src;
}

template <class T>
__global__ void __launch_bounds__(1024) k_batch(BatchArgs a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t next;
    __shared__ LayerCoefs<T> lc;
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smem_raw);
    const T *coef = static_cast<const T *>(a.coef);
    T *probs = static_cast<T *>(a.probs);
    cplx<T> *slot = static_cast<cplx<T> *>(a.arena) + uint64_t(blockIdx.x) * 2 * a.slot_amps;
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(a.counter, 1u);
        __syncthreads();
        const uint32_t w = next;
        __syncthreads();
        if (w >= a.ninst) break;
        const uint32_t id = a.order[w];
        const InstDesc d = a.inst[id];
        if (d.n <= a.tile_log2) {
            run_small<T>(sm, lc, d, coef);
            // the terms go after the state when it fills at most half the tile
            T *nrm = d.n < a.tile_log2 ? reinterpret_cast<T *>(sm + (uint64_t(1) << d.n)) : nullptr;
            finish_instance<T>(sm, nrm, d, probs, a.norms + d.norms);
        } else {
            const cplx<T> *fin = run_big<T>(sm, lc, d, coef, slot, slot + a.slot_amps, a.tile_log2);
            finish_big<T>(fin, sm, a.tile_log2, d, probs, a.norms + d.norms);
        }
    }
}

// The sampling CDFs, after k_batch, one instance per warp (instance
// cdf_order[w] for warp w).  A uniform's outcome is the first index whose
// running double sum of |a|^2 terms reaches it, index 0 when none does
// (measure.cpp:60-78, :164-188).  The running sum s is exact at all times:
//   - while s is normal, in binade e, a round of 32 x CDF_RUN terms runs in
//     parallel: each lane takes CDF_RUN consecutive terms, a warp scan of
//     their grid-step transducers (replay.cuh) gives every lane the grid
//     position where its run starts, and each lane walks its run; the round
//     stops before the first term whose sum would leave the binade (or that
//     is too big for it), which is then added on its own with one FP64 add;
//   - while s is zero, runs of zero terms are skipped 32 at a time, and
//     while it is subnormal, terms are added one at a time.
// After every term, all uniforms the sum has reached take that term's index,
// so the outcomes are the sequential merge's.
constexpr unsigned CDF_RUN = 16;
constexpr uint64_t CDF_NONE = ~uint64_t(0);

__device__ __forceinline__ Tx shfl_up_tx(const Tx &t, unsigned off)
{
    Tx r;
    r.d[0] = __shfl_up_sync(0xFFFFFFFFu, (unsigned long long)t.d[0], off);
    r.d[1] = __shfl_up_sync(0xFFFFFFFFu, (unsigned long long)t.d[1], off);
    return r;
}

__global__ void __launch_bounds__(CDF_THREADS) k_batch_cdf(BatchArgs a)
{
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned lane = threadIdx.x & 31;
    if (w >= a.ninst) return;                             // whole warps
    const uint32_t id = a.cdf_order[w];
    const InstDesc d = a.inst[id];
    const double *__restrict__ nr = a.norms + d.norms;
    const double *__restrict__ u = a.usorted + uint64_t(id) * a.nshots;
    uint64_t *__restrict__ out = a.shots + d.shots;
    const uint64_t dim = uint64_t(1) << d.n;
    const uint32_t ns = a.nshots;
    uint32_t k = 0;                                       // next uniform
    double s = 0.0;                                       // the sum of terms 0..i-1
    uint64_t i = 0;                                       // next term
    // every uniform the sum s has reached takes index `idx`
    auto consume = [&](uint64_t idx) {
        while (k < ns && cdf_reached(u[k], s)) {
            if (lane == 0) out[k] = idx;
            k++;
        }
    };
    while (i < dim && k < ns) {
        const int e = binade(s);
        if (e < fp_traits<double>::EMIN) {
            if (__double_as_longlong(s) == 0) {
                // zero so far: skip to the first nonzero term of the next 32
                const uint64_t j = i + lane;
                const unsigned nz = __ballot_sync(0xFFFFFFFFu, j < dim && __double_as_longlong(nr[j]) != 0);
                consume(i);                               // u == 0 is reached at term i
                if (!nz) {
                    i = i + 32 < dim ? i + 32 : dim;
                    continue;
                }
                i += unsigned(__ffs(nz) - 1);
            }
            s = __dadd_rn(s, nr[i]);                      // subnormal (or zero) sum: one term
            consume(i);
            i++;
            continue;
        }
        // a round of terms [i, end) in binade e
        const uint64_t m0 = grid_pos(s);
        const uint64_t end = i + 32 * CDF_RUN < dim ? i + 32 * CDF_RUN : dim;
        const uint64_t base = i + uint64_t(lane) * CDF_RUN;
        const unsigned len = base < end ? unsigned(end - base < CDF_RUN ? end - base : CDF_RUN) : 0u;
        auto run = [nr, base](unsigned r) { return nr[base + r]; };
        bool big = false;
        const Tx mine = run_effect<double>(run, len, e, big);
        Tx incl = mine;
        for (unsigned off = 1; off < 32; off <<= 1) {
            const Tx o = shfl_up_tx(incl, off);
            if (lane >= off) incl = tx_then(o, incl);
        }
        Tx excl = shfl_up_tx(incl, 1);
        if (lane == 0) excl = tx_identity();
        const uint64_t pos0 = m0 + excl.d[m0 & 1];        // grid position before this lane's run
        uint64_t pos = pos0;
        const unsigned walked = run_walk<double>(run, len, e, pos);
        uint64_t bad = walked < len ? base + walked : CDF_NONE;
        for (unsigned off = 16; off; off >>= 1) {
            const uint64_t o = __shfl_xor_sync(0xFFFFFFFFu, (unsigned long long)bad, off);
            bad = o < bad ? o : bad;
        }
        const uint64_t stop = bad == CDF_NONE ? end : bad;
        // the position after term stop - 1: where the lane holding `stop`
        // stopped, or where the lane holding the round's last term ended
        const uint64_t last = bad == CDF_NONE ? end - 1 : stop;
        const unsigned holder = unsigned((last - i) / CDF_RUN);
        const uint64_t pend = __shfl_sync(0xFFFFFFFFu, (unsigned long long)pos, holder);
        // uniforms reached inside [i, stop): the first term whose position
        // reaches the uniform's grid target
        const bool live = len && base < stop;
        while (k < ns) {
            const uint64_t tgt = grid_ceil<double>(u[k], e);
            if (tgt > pend) break;
            const unsigned hit = __ballot_sync(0xFFFFFFFFu, live && pos >= tgt);
            if (!hit) break;                              // not reached: pend >= tgt rules it out
            const unsigned L = unsigned(__ffs(hit) - 1);
            uint64_t j = 0;
            if (lane == L) j = base + run_find<double>(run, len, e, pos0, tgt);
            j = __shfl_sync(0xFFFFFFFFu, (unsigned long long)j, L);
            if (lane == 0) out[k] = j;
            k++;
        }
        s = grid_at<double>(pend, e);
        i = stop;
        if (bad != CDF_NONE) {
            s = __dadd_rn(s, nr[i]);                      // the term that leaves the binade
            consume(i);
            i++;
        }
    }
    for (; k < ns; k++)
        if (lane == 0) out[k] = 0;                        // above the total: index 0
}

}  // namespace
}  // namespace qslc

using namespace qslc;

// One launch shape of the persistent kernel.
struct BatchShape {
    unsigned threads = 1024;
    unsigned tile_log2 = 13;
    unsigned ctas_per_sm = 1;
};

struct qslc_batch {
    int dtype = QSLC_C128;
    uint32_t ninst = 0, nshots = 0, nmax = 0;
    std::vector<InstDesc> inst;
    std::vector<uint32_t> order, cdf_order;
    uint64_t ncoef = 0, nprobs = 0, nshot_total = 0, nnorm_total = 0;
    cudaStream_t stream = nullptr;
    void *d_inst = nullptr, *d_order = nullptr, *d_counter = nullptr, *d_coef = nullptr;
    void *d_probs = nullptr, *d_u = nullptr, *d_shots = nullptr, *d_arena = nullptr;
    void *d_norms = nullptr, *d_cdf_order = nullptr;
    uint64_t arena_bytes = 0, slot_amps = 0;
    BatchShape shape;
    unsigned grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t runs = 0;
};

namespace {

// The arena holds two buffers of 2^nmax amplitudes per CTA; beyond this
// many bytes the grid shrinks instead.
constexpr uint64_t ARENA_CAP = uint64_t(64) << 30;

size_t amp_bytes(int dtype) { return dtype == QSLC_C128 ? 16 : 8; }

void drop_graph(qslc_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

void batch_free(qslc_batch *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    drop_graph(b);
    for (void *p : {b->d_inst, b->d_order, b->d_counter, b->d_coef, b->d_probs, b->d_u, b->d_shots,
                    b->d_arena, b->d_norms, b->d_cdf_order})
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Whether a shape can run this batch: the tile must fit a CTA's shared
// memory and cover at least half of the largest instance's qubits.
bool shape_fits(const qslc_batch *b, const BatchShape &s)
{
    const size_t tile = (size_t(1) << s.tile_log2) * amp_bytes(b->dtype);
    if (tile * s.ctas_per_sm + 16 * 1024 * s.ctas_per_sm > 224 * 1024) return false;
    if (s.threads * s.ctas_per_sm > 1024) return false;   // registers: 64 K per SM, up to 64 a thread
    if (b->nmax > 2 * s.tile_log2) return false;
    return true;
}

// (Re)capture the graph for shape `s`: grid, arena size, kernel attributes.
template <class T>
int capture(qslc_batch *b, const BatchShape &s)
{
    drop_graph(b);
    const size_t ab = amp_bytes(b->dtype);
    const size_t smem = (size_t(1) << s.tile_log2) * ab;
    b->slot_amps = b->nmax > s.tile_log2 ? (uint64_t(1) << b->nmax) : 0;
    unsigned grid = sm_count() * s.ctas_per_sm;
    if (b->slot_amps) {
        const uint64_t slot = 2 * b->slot_amps * ab;
        grid = unsigned(std::min<uint64_t>(grid, std::max<uint64_t>(1, ARENA_CAP / slot)));
    }
    grid = std::min<unsigned>(grid, b->ninst);
    const uint64_t need = uint64_t(grid) * 2 * b->slot_amps * ab;
    if (need > b->arena_bytes) {
        if (b->d_arena) cudaFree(b->d_arena);
        b->d_arena = nullptr;
        b->arena_bytes = 0;
        if (cudaMalloc(&b->d_arena, std::max<uint64_t>(need, 16)) != cudaSuccess) {
            cudaGetLastError();
            return fail(QSLC_EOOM, "out of device memory for the batch arena");
        }
        b->arena_bytes = need;
    }
    QSLC_CUDA(cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    BatchArgs a;
    a.inst = static_cast<const InstDesc *>(b->d_inst);
    a.order = static_cast<const uint32_t *>(b->d_order);
    a.ninst = b->ninst;
    a.counter = static_cast<unsigned *>(b->d_counter);
    a.coef = b->d_coef;
    a.probs = b->d_probs;
    a.usorted = static_cast<const double *>(b->d_u);
    a.shots = static_cast<uint64_t *>(b->d_shots);
    a.nshots = b->nshots;
    a.norms = static_cast<double *>(b->d_norms);
    a.cdf_order = static_cast<const uint32_t *>(b->d_cdf_order);
    a.arena = b->d_arena;
    a.slot_amps = b->slot_amps;
    a.tile_log2 = s.tile_log2;
    QSLC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), b->stream);
    k_batch<T><<<grid, s.threads, smem, b->stream>>>(a);
    k_batch_cdf<<<(b->ninst + CDF_THREADS / 32 - 1) / (CDF_THREADS / 32), CDF_THREADS, 0, b->stream>>>(a);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    b->graph = g;
    QSLC_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    b->shape = s;
    b->grid = grid;
    return QSLC_OK;
}

int capture_any(qslc_batch *b, const BatchShape &s)
{
    return b->dtype == QSLC_C128 ? capture<double>(b, s) : capture<float>(b, s);
}

// f(i) for every i in [0, n) on the host's cores: instance i goes to thread
// i mod T, so instances of every size spread over the threads.  Each f(i)
// touches only instance i's data.
template <class F>
void host_parallel(uint32_t n, F &&f)
{
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::min<unsigned>(std::max<unsigned>(nt, 1u), 32u);
    if (nt < 2 || n < 256) {
        for (uint32_t i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(nt);
    for (unsigned t = 0; t < nt; t++)
        pool.emplace_back([&f, n, nt, t] {
            for (uint32_t i = t; i < n; i += nt) f(i);
        });
    for (auto &th : pool) th.join();
}

// Coefficients exactly as the reference computes them (gates.cpp:154-155,
// :185-186: Fp cos/sin of Fp(angle)/2) and each instance's uniforms sorted
// (in Fp, as the reference draws them), uploaded; `perm` maps sorted
// positions back to the caller's order.
template <class T>
int upload_inputs(qslc_batch *b, const double *angles, const double *u, std::vector<uint32_t> &perm)
{
    std::vector<T> coef(b->ncoef);
    // instance i's angles start at 2 x (its coefficients' offset) / 4
    host_parallel(b->ninst, [&](uint32_t i) {
        const InstDesc &d = b->inst[i];
        const double *ai = angles + d.coef / 2;
        for (uint64_t k = 0; k < uint64_t(d.L) * d.n; k++) {
            const T ry = T(ai[2 * k]), rz = T(ai[2 * k + 1]);
            T *c = &coef[d.coef + 4 * k];
            c[0] = T(std::cos(ry / 2));
            c[1] = T(std::sin(ry / 2));
            c[2] = T(std::cos(rz / 2));
            c[3] = T(std::sin(rz / 2));
        }
    });
    const uint32_t ns = b->nshots;
    std::vector<double> us(uint64_t(b->ninst) * ns);
    perm.resize(uint64_t(b->ninst) * ns);
    host_parallel(b->ninst, [&](uint32_t i) {
        uint32_t *pm = perm.data() + uint64_t(i) * ns;
        const double *ui = u + uint64_t(i) * ns;
        std::iota(pm, pm + ns, 0u);
        std::sort(pm, pm + ns, [&](uint32_t x, uint32_t y) { return ui[x] < ui[y]; });
        for (uint32_t k = 0; k < ns; k++) {
            double v = ui[pm[k]];
            if (b->dtype == QSLC_C64) v = double(float(v));   // the reference draws Fp uniforms
            us[uint64_t(i) * ns + k] = v;
        }
    });
    QSLC_CUDA(cudaMemcpyAsync(b->d_coef, coef.data(), coef.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream));
    QSLC_CUDA(cudaMemcpyAsync(b->d_u, us.data(), us.size() * 8, cudaMemcpyHostToDevice, b->stream));
    QSLC_CUDA(cudaStreamSynchronize(b->stream));
    return QSLC_OK;
}

int upload_any(qslc_batch *b, const double *angles, const double *u, std::vector<uint32_t> &perm)
{
    return b->dtype == QSLC_C128 ? upload_inputs<double>(b, angles, u, perm)
                                 : upload_inputs<float>(b, angles, u, perm);
}

template <class T>
int download(qslc_batch *b, const std::vector<uint32_t> &perm, double *probs, uint64_t *shots)
{
    std::vector<T> pr(b->nprobs);
    std::vector<uint64_t> sh(b->nshot_total);
    QSLC_CUDA(cudaMemcpyAsync(pr.data(), b->d_probs, pr.size() * sizeof(T), cudaMemcpyDeviceToHost, b->stream));
    QSLC_CUDA(cudaMemcpyAsync(sh.data(), b->d_shots, sh.size() * 8, cudaMemcpyDeviceToHost, b->stream));
    QSLC_CUDA(cudaStreamSynchronize(b->stream));
    QSLC_CUDA(cudaGetLastError());
    for (uint64_t i = 0; i < b->nprobs; i++) probs[i] = double(pr[i]);
    const uint32_t ns = b->nshots;
    host_parallel(b->ninst, [&](uint32_t i) {
        for (uint32_t k = 0; k < ns; k++)
            shots[uint64_t(i) * ns + perm[uint64_t(i) * ns + k]] = sh[b->inst[i].shots + k];
    });
    return QSLC_OK;
}

// The launch shapes the autotuner measures: threads per CTA, a tile of
// 64 or 128 KB, one or two CTAs per SM.
std::vector<BatchShape> candidates(const qslc_batch *b)
{
    const unsigned k128 = b->dtype == QSLC_C128 ? 13 : 14;
    std::vector<BatchShape> out;
    for (unsigned th : {512u, 1024u})
        for (const auto &tc : {std::pair<unsigned, unsigned>{k128 - 1, 2u}, {k128 - 1, 1u}, {k128, 1u}}) {
            BatchShape s;
            s.threads = th;
            s.tile_log2 = tc.first;
            s.ctas_per_sm = tc.second;
            if (shape_fits(b, s)) out.push_back(s);
        }
    return out;
}

}  // namespace

extern "C" int qslc_batch_create(int dtype, uint32_t ninst, const uint32_t *nqubits,
                                 const uint32_t *nlayers, uint32_t nshots, qslc_batch **out)
{
    QSLC_ENTRY("qslc_batch_create");
    if (!out || !nqubits || !nlayers || ninst == 0) return fail(QSLC_EINVAL, "bad batch arguments");
    *out = nullptr;
    if (dtype != QSLC_C128 && dtype != QSLC_C64) return fail(QSLC_EINVAL, "unknown dtype");
    auto *b = new qslc_batch();
    b->dtype = dtype;
    b->ninst = ninst;
    b->nshots = nshots;
    b->inst.resize(ninst);
    for (uint32_t i = 0; i < ninst; i++) {
        if (nqubits[i] < 2 || nqubits[i] > uint32_t(MAX_Q)) {
            delete b;
            return fail(QSLC_EINVAL, "batch instances take 2..26 qubits");
        }
        InstDesc &d = b->inst[i];
        d.n = nqubits[i];
        d.L = nlayers[i];
        d.coef = b->ncoef;
        d.probs = b->nprobs;
        d.shots = b->nshot_total;
        d.norms = b->nnorm_total;
        b->ncoef += uint64_t(d.L) * d.n * 4;
        b->nnorm_total += uint64_t(1) << d.n;
        b->nprobs += 2 * uint64_t(d.n);
        b->nshot_total += nshots;
        b->nmax = std::max(b->nmax, d.n);
    }
    // largest instances first, so the long ones start early
    b->order.resize(ninst);
    std::iota(b->order.begin(), b->order.end(), 0u);
    std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t x, uint32_t y) {
        return (uint64_t(b->inst[x].L) << b->inst[x].n) > (uint64_t(b->inst[y].L) << b->inst[y].n);
    });
    // the CDF walks: one instance per thread, a warp's instances of about
    // the same length
    b->cdf_order.resize(ninst);
    std::iota(b->cdf_order.begin(), b->cdf_order.end(), 0u);
    std::stable_sort(b->cdf_order.begin(), b->cdf_order.end(),
                     [&](uint32_t x, uint32_t y) { return b->inst[x].n > b->inst[y].n; });
    const size_t fb = dtype == QSLC_C128 ? 8 : 4;
    int rc = QSLC_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (rc) return;
        if (cudaMalloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
            cudaGetLastError();
            rc = fail(QSLC_EOOM, "out of device memory for the batch");
        }
    };
    alloc(&b->d_inst, ninst * sizeof(InstDesc));
    alloc(&b->d_order, ninst * 4);
    alloc(&b->d_counter, 16);
    alloc(&b->d_coef, b->ncoef * fb);
    alloc(&b->d_probs, b->nprobs * fb);
    alloc(&b->d_u, b->nshot_total * 8);
    alloc(&b->d_shots, b->nshot_total * 8);
    alloc(&b->d_norms, b->nnorm_total * 8);
    alloc(&b->d_cdf_order, ninst * 4);
    if (!rc && cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "stream creation failed");
    if (!rc && cudaMemcpy(b->d_inst, b->inst.data(), ninst * sizeof(InstDesc), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "upload failed");
    if (!rc && cudaMemcpy(b->d_order, b->order.data(), ninst * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "upload failed");
    if (!rc && cudaMemcpy(b->d_cdf_order, b->cdf_order.data(), ninst * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "upload failed");
    if (!rc) {
        const auto c = candidates(b);
        if (c.empty()) rc = fail(QSLC_EINVAL, "no launch shape fits the largest instance");
        else rc = capture_any(b, c.back());    // 1024 threads, one CTA per SM
    }
    if (rc) {
        batch_free(b);
        return rc;
    }
    *out = b;
    return QSLC_OK;
}

extern "C" int qslc_batch_run(qslc_batch *b, const double *angles, const double *uniforms,
                              double *probs, uint64_t *shots)
{
    QSLC_ENTRY("qslc_batch_run");
    if (!b || !angles || !probs || (!uniforms && b->nshots) || (!shots && b->nshots))
        return fail(QSLC_EINVAL, "null pointer");
    std::vector<uint32_t> perm;
    int rc = upload_any(b, angles, uniforms, perm);
    if (rc) return rc;
    QSLC_CUDA(cudaGraphLaunch(b->exec, b->stream));
    rc = b->dtype == QSLC_C128 ? download<double>(b, perm, probs, shots) : download<float>(b, perm, probs, shots);
    if (!rc) b->runs++;
    return rc;
}

extern "C" int qslc_batch_autotune(qslc_batch *b, const double *angles, const double *uniforms,
                                   double *best_ms)
{
    QSLC_ENTRY("qslc_batch_autotune");
    if (!b || !angles || (!uniforms && b->nshots)) return fail(QSLC_EINVAL, "null pointer");
    std::vector<uint32_t> perm;
    int rc = upload_any(b, angles, uniforms, perm);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    QSLC_CUDA(cudaEventCreate(&e0));
    QSLC_CUDA(cudaEventCreate(&e1));
    BatchShape best = b->shape;
    float best_t = -1.f;
    for (const BatchShape &s : candidates(b)) {
        rc = capture_any(b, s);
        if (rc) break;
        QSLC_CUDA(cudaGraphLaunch(b->exec, b->stream));        // warm-up
        QSLC_CUDA(cudaEventRecord(e0, b->stream));
        QSLC_CUDA(cudaGraphLaunch(b->exec, b->stream));
        QSLC_CUDA(cudaEventRecord(e1, b->stream));
        QSLC_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        QSLC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (best_t < 0.f || ms < best_t) {
            best_t = ms;
            best = s;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) rc = capture_any(b, best);
    if (!rc && best_ms) *best_ms = double(best_t);
    return rc;
}

extern "C" int qslc_batch_set_shape(qslc_batch *b, unsigned threads, unsigned tile_log2,
                                    unsigned ctas_per_sm)
{
    QSLC_ENTRY("qslc_batch_set_shape");
    if (!b) return fail(QSLC_EINVAL, "null batch");
    BatchShape s;
    s.threads = threads;
    s.tile_log2 = tile_log2;
    s.ctas_per_sm = ctas_per_sm;
    for (const BatchShape &c : candidates(b))
        if (c.threads == s.threads && c.tile_log2 == s.tile_log2 && c.ctas_per_sm == s.ctas_per_sm)
            return capture_any(b, s);
    return fail(QSLC_EINVAL, "not one of the launch shapes this batch can take");
}

extern "C" int qslc_batch_shape(const qslc_batch *b, unsigned *threads, unsigned *tile_log2,
                                unsigned *ctas_per_sm, unsigned *grid)
{
    QSLC_ENTRY("qslc_batch_shape");
    if (!b) return fail(QSLC_EINVAL, "null batch");
    if (threads) *threads = b->shape.threads;
    if (tile_log2) *tile_log2 = b->shape.tile_log2;
    if (ctas_per_sm) *ctas_per_sm = b->shape.ctas_per_sm;
    if (grid) *grid = b->grid;
    return QSLC_OK;
}

extern "C" int qslc_batch_destroy(qslc_batch *b)
{
    batch_free(b);
    return QSLC_OK;
}
