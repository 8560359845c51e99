// np.cu -- the number-preserving (NP) backend on a compressed layout.
//
// qsl's NP simulator keeps the full 2^n vector and walks lookup tables of
// fixed-weight integers (src/qubits/np/np.cpp:168-181, misc.cpp:75-90).
// Here only the C(n, w) amplitudes of weight w are stored, in ascending
// order of their basis index, so amplitude y lives at slot rank(y): the
// number of weight-w integers below y, which the combinatorial number
// system gives as sum over the set bits of y, the t-th lowest at position
// p_t, of C(p_t, t).
//
// The device holds the same five pattern tables the reference builds
// ({n-1, w-1}, {n-2, w-1}, {n-2, w-2}, {n-1, w}, {n, w}), produced in
// parallel by unranking, plus a table of partial ranks per 8-bit chunk:
// rank(y) = sum over chunks c of R[c][popc(y below chunk c)][byte c of y].
// A gate thread takes one pattern x, inserts the gate's qubit bits exactly
// as the reference does (np/gates.cpp:39-51, :127-147) and ranks the
// resulting basis indices to find their slots.  The {n, w} table doubles as
// the slot -> basis index map used by measurement.
#include "gatemath.cuh"
#include "seqsum.cuh"
#include "np_host.hpp"

#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace qslc {

namespace {

constexpr int NP_MAXN = 32;   // the reference's next() is 32-bit (misc.cpp:36)
__constant__ uint32_t c_binom[NP_MAXN + 1][NP_MAXN + 1];
#define h_binom (host_binom().v)

// Partial-rank table, [chunk 0..3][k 0..32][byte value]: 4*33*256 entries.
constexpr int RT_K = NP_MAXN + 1;
uint32_t *d_rank_tab = nullptr;
std::once_flag g_np_once;
int g_np_status = QSLC_OK;

__host__ __device__ __forceinline__ uint32_t binom_dev(unsigned n, unsigned k)
{
#ifdef __CUDA_ARCH__
    return (k > n) ? 0u : c_binom[n][k];
#else
    return (k > n) ? 0u : uint32_t(h_binom[n][k]);
#endif
}

__device__ __forceinline__ uint32_t rank_dev(const uint32_t *__restrict__ rt, uint32_t y)
{
    uint32_t r = 0;
    unsigned k = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        uint32_t byte = (y >> (8 * c)) & 0xFFu;
        r += __ldg(rt + (c * RT_K + k) * 256 + byte);
        k += __popc(byte);
    }
    return r;
}

// the r-th (0-based) integer of `ones` set bits in `len` bits, ascending
__device__ __forceinline__ uint32_t unrank_dev(uint64_t r, unsigned len, unsigned ones)
{
    uint32_t x = 0;
    unsigned t = ones;
    for (int p = int(len) - 1; p >= 0 && t > 0; p--) {
        uint32_t c = binom_dev(unsigned(p), t);
        if (c <= r) {
            x |= 1u << p;
            r -= c;
            t--;
        }
    }
    return x;
}

__global__ void k_np_build_table(uint32_t *__restrict__ tab, uint64_t count, unsigned len,
                                 unsigned ones)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t r = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; r < count; r += stride)
        tab[r] = unrank_dev(r, len, ones);
}

__host__ __device__ __forceinline__ uint32_t ins_bit(uint32_t x, unsigned t, uint32_t v)
{
    uint32_t lower = x & ((1u << t) - 1u);
    return lower | (v << t) | ((x & ~((1u << t) - 1u)) << 1);
}
__host__ __device__ __forceinline__ uint32_t ins00(uint32_t x, unsigned lo, unsigned hi)
{
    // lower + (mid << 1) + (upper << 2), np/gates.cpp:127-147
    uint32_t small_bit = 1u << lo, large_bit = 1u << hi;
    uint32_t lower_mask = small_bit - 1u;
    uint32_t mid_mask = ((large_bit >> 1) - 1u) ^ lower_mask;
    uint32_t upper_mask = ~(lower_mask | mid_mask);
    return (x & lower_mask) + ((x & mid_mask) << 1) + ((x & upper_mask) << 2);
}

// Items per thread and grid-stride iteration of the NP sweeps.  Each item
// waits on two dependent reads (its pattern, then its amplitude), so these
// sweeps are bound by memory latency rather than arithmetic; two items
// measured faster than three or four on the 28-qubit weight-14 circuit
// (6964, 6758 and 6466 gates/s).
#ifndef QSLC_NP_ITEMS
#define QSLC_NP_ITEMS 2
#endif
constexpr int NP_ITEMS = QSLC_NP_ITEMS;

enum NPKind {
    NP_PHASE1, NP_NEG1, NP_RZ0,                 // one-qubit, single amplitude
    NP_CZ, NP_CPHASE, NP_CRZ01,                 // two-qubit, single amplitude
    NP_SWAP, NP_RX, NP_RY, NP_H                 // two-qubit pairs
};

// Single-amplitude updates (np/gates.cpp:53-55, :77-78, :104-106, :148-149,
// :183-185, :229-231).  NP_ITEMS items per grid-stride iteration; `pat`
// chooses per item how each of the two outputs is computed (gatemath.cuh).
template <class T, int K, unsigned CPAT = PAT_RUNTIME>
__global__ void QSLC_SWEEP_BOUNDS k_np_single(cplx<T> *__restrict__ st,
                                                   const uint32_t *__restrict__ tab, uint64_t count,
                                                   const uint32_t *__restrict__ rt, unsigned t1,
                                                   unsigned t2, uint32_t addbits, Coef<T> k,
                                                   unsigned pat)
{
    using R = rn<T>;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    // the pattern-table entries of the next iteration are read while this
    // iteration's amplitudes are in flight, so the two dependent DRAM reads
    // of an item (its pattern, then its amplitude) overlap across iterations
    const uint64_t j0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    uint32_t xn[NP_ITEMS];
#pragma unroll
    for (int r = 0; r < NP_ITEMS; r++) xn[r] = (j0 + r * stride < count) ? tab[j0 + r * stride] : 0u;
    for (uint64_t j = j0; j < count; j += NP_ITEMS * stride) {
        uint32_t slot[NP_ITEMS];
        cplx<T> a[NP_ITEMS];
        uint32_t xc[NP_ITEMS];
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) xc[r] = xn[r];
        const uint64_t jn = j + NP_ITEMS * stride;
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++)
            if (jn + r * stride < count) xn[r] = tab[jn + r * stride];
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) {
            if (j + r * stride < count) {
                const uint32_t x = xc[r];
                uint32_t y;
                if constexpr (K == NP_PHASE1 || K == NP_NEG1 || K == NP_RZ0)
                    y = ins_bit(x, t1, 0) | addbits;
                else
                    y = ins00(x, t1, t2) | addbits;
                slot[r] = rank_dev(rt, y);
                a[r] = st[slot[r]];
            }
        }
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) {
            if (j + r * stride >= count) continue;
            const unsigned md = (pt >> (8 * r)) & 0xFFu;
            const T re = a[r].x, im = a[r].y;
            if constexpr (K == NP_NEG1 || K == NP_CZ) {
                a[r].x = R::mul(re, T(-1));
                a[r].y = R::mul(im, T(-1));
            } else if constexpr (K == NP_RZ0 || K == NP_CRZ01) {
                // cos*re + sin*im, cos*im - sin*re
                a[r].x = dot2m<T, false>(mode_of(md, 0), re, k.c, k.kc, k.mc, im, k.s, k.ks, k.ms);
                a[r].y = dot2m<T, true>(mode_of(md, 1), im, k.c, k.kc, k.mc, re, k.s, k.ks, k.ms);
            } else {
                // phase * amplitude: cos*re - sin*im, cos*im + sin*re
                a[r].x = dot2m<T, true>(mode_of(md, 0), re, k.c, k.kc, k.mc, im, k.s, k.ks, k.ms);
                a[r].y = dot2m<T, false>(mode_of(md, 1), im, k.c, k.kc, k.mc, re, k.s, k.ks, k.ms);
            }
            st[slot[r]] = a[r];
        }
    }
}

// Pair updates over table {n-2, w-1} (np/gates.cpp:236-415).
template <class T, int K, unsigned CPAT = PAT_RUNTIME>
__global__ void QSLC_SWEEP_BOUNDS k_np_pair(cplx<T> *__restrict__ st,
                                                 const uint32_t *__restrict__ tab, uint64_t count,
                                                 const uint32_t *__restrict__ rt, unsigned lo,
                                                 unsigned hi, uint32_t b1, uint32_t b2, Coef<T> k,
                                                 unsigned pat)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const unsigned pt = CPAT == PAT_RUNTIME ? pat : CPAT;
    // next iteration's pattern-table entries read ahead, as in k_np_single
    const uint64_t j0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    uint32_t xn[NP_ITEMS];
#pragma unroll
    for (int r = 0; r < NP_ITEMS; r++) xn[r] = (j0 + r * stride < count) ? tab[j0 + r * stride] : 0u;
    for (uint64_t j = j0; j < count; j += NP_ITEMS * stride) {
        uint32_t s1[NP_ITEMS], s2[NP_ITEMS];
        cplx<T> a0[NP_ITEMS], a1[NP_ITEMS];
        uint32_t xc[NP_ITEMS];
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) xc[r] = xn[r];
        const uint64_t jn = j + NP_ITEMS * stride;
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++)
            if (jn + r * stride < count) xn[r] = tab[jn + r * stride];
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) {
            if (j + r * stride < count) {
                const uint32_t base = ins00(xc[r], lo, hi);
                s1[r] = rank_dev(rt, base | b1);
                s2[r] = rank_dev(rt, base | b2);
                a0[r] = st[s1[r]];
                a1[r] = st[s2[r]];
            }
        }
#pragma unroll
        for (int r = 0; r < NP_ITEMS; r++) {
            if (j + r * stride >= count) continue;
            const unsigned md = (pt >> (8 * r)) & 0xFFu;
            const unsigned E0 = mode_of(md, 0), E1 = mode_of(md, 1), E2 = mode_of(md, 2), E3 = mode_of(md, 3);
            const cplx<T> p = a0[r], q = a1[r];
            cplx<T> r0, r1;
            if constexpr (K == NP_SWAP) {
                r0 = q;
                r1 = p;
            } else if constexpr (K == NP_RX) {       // :316-321
                r0.x = dot2m<T, false>(E0, p.x, k.c, k.kc, k.mc, q.y, k.s, k.ks, k.ms);
                r0.y = dot2m<T, true>(E1, p.y, k.c, k.kc, k.mc, q.x, k.s, k.ks, k.ms);
                r1.x = dot2m<T, false>(E2, q.x, k.c, k.kc, k.mc, p.y, k.s, k.ks, k.ms);
                r1.y = dot2m<T, true>(E3, q.y, k.c, k.kc, k.mc, p.x, k.s, k.ks, k.ms);
            } else if constexpr (K == NP_RY) {       // :366-371
                r0.x = dot2m<T, true>(E0, p.x, k.c, k.kc, k.mc, q.x, k.s, k.ks, k.ms);
                r0.y = dot2m<T, true>(E1, p.y, k.c, k.kc, k.mc, q.y, k.s, k.ks, k.ms);
                r1.x = dot2m<T, false>(E2, p.x, k.s, k.ks, k.ms, q.x, k.c, k.kc, k.mc);
                r1.y = dot2m<T, false>(E3, p.y, k.s, k.ks, k.ms, q.y, k.c, k.kc, k.mc);
            } else {                                 // NP_H, :409-412
                r0.x = hdiv<T, false>(E0 != MD_F, p.x, q.x, k);
                r0.y = hdiv<T, false>(E1 != MD_F, p.y, q.y, k);
                r1.x = hdiv<T, true>(E2 != MD_F, p.x, q.x, k);
                r1.y = hdiv<T, true>(E3 != MD_F, p.y, q.y, k);
            }
            st[s1[r]] = r0;
            st[s2[r]] = r1;
        }
    }
}

// collapse (np/measure.cpp:32-70): scale over table {n-1, w-o} with bit t
// = o inserted, zero over {n-1, w-(o^1)} with bit t = o^1.
template <class T>
__global__ void __launch_bounds__(256) k_np_scale(cplx<T> *__restrict__ st,
                                                  const uint32_t *__restrict__ tab, uint64_t count,
                                                  const uint32_t *__restrict__ rt, unsigned t,
                                                  uint32_t v, T factor, int zero)
{
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t j = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; j < count; j += stride) {
        const uint32_t slot = rank_dev(rt, ins_bit(tab[j], t, v));
        cplx<T> a = st[slot];
        if (zero) {
            a.x = T(0);
            a.y = T(0);
        } else {
            a.x = rn<T>::mul(a.x, factor);
            a.y = rn<T>::mul(a.y, factor);
        }
        st[slot] = a;
    }
}

// Measurement producers over the compressed layout.  Slot j holds basis
// index basis[j] (the {n, w} table); zero terms leave a running sum
// unchanged, so prob's sum over the slots with bit t == o, in slot order,
// is the reference's sum over table {n-1, w-o} (np/measure.cpp:141-168).
template <class T>
struct ProdNPMask {
    const cplx<T> *amps;
    const uint32_t *basis;
    unsigned t;
    uint32_t o;
    __device__ __forceinline__ uint64_t index(uint64_t j) const { return basis[j]; }
    __device__ __forceinline__ T p(uint64_t j) const
    {
        if (((basis[j] >> t) & 1u) != o) return T(0);
        cplx<T> a = amps[j];
        return norm2_rn(a.x, a.y);
    }
};
template <class T>
struct ProdNPAll {
    const cplx<T> *amps;
    const uint32_t *basis;
    __device__ __forceinline__ uint64_t index(uint64_t j) const { return basis[j]; }
    __device__ __forceinline__ T p(uint64_t j) const
    {
        cplx<T> a = amps[j];
        return norm2_rn(a.x, a.y);
    }
};

int init_once()
{
    static uint32_t tmp[NP_MAXN + 1][NP_MAXN + 1];
    for (int n = 0; n <= NP_MAXN; n++)
        for (int k = 0; k <= NP_MAXN; k++) tmp[n][k] = uint32_t(k <= n ? h_binom[n][k] : 0);
    QSLC_CUDA(cudaMemcpyToSymbol(c_binom, tmp, sizeof(tmp)));
    std::vector<uint32_t> rt(size_t(4) * RT_K * 256, 0);
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < RT_K; k++)
            for (int v = 0; v < 256; v++) {
                uint64_t r = 0;
                int i = 0;
                for (int b = 0; b < 8; b++)
                    if (v & (1 << b)) {
                        i++;
                        int pos = 8 * c + b, tt = k + i;
                        if (tt <= pos) r += h_binom[pos][tt];
                    }
                rt[(size_t(c) * RT_K + k) * 256 + v] = uint32_t(r);
            }
    QSLC_CUDA(cudaMalloc(&d_rank_tab, rt.size() * 4));
    QSLC_CUDA(cudaMemcpy(d_rank_tab, rt.data(), rt.size() * 4, cudaMemcpyHostToDevice));
    return QSLC_OK;
}

}  // namespace

// index of table {len, ones} in NPTables::tab
enum { T_N1W1 = 0, T_N2W1 = 1, T_N2W2 = 2, T_N1W = 3, T_NW = 4 };

uint64_t np_choose(unsigned n, unsigned k) { return choose_u64(n, k); }

uint64_t np_rank_host(uint64_t y) { return rank_of(y); }

int np_init_tables()
{
    std::call_once(g_np_once, [] { g_np_status = init_once(); });
    return g_np_status;
}

static NPTables *tables_of(qslc_state *s)
{
    if (!s->npt) s->npt = new NPTables();
    return s->npt;
}

void np_release(qslc_state *s)
{
    if (!s->npt) return;
    for (auto *p : s->npt->tab)
        if (p) cudaFree(p);
    delete s->npt;
    s->npt = nullptr;
}

int np_prepare(qslc_state *s, unsigned w)
{
    int rc = np_init_tables();
    if (rc) return rc;
    NPTables *tb = tables_of(s);
    if (tb->n == s->n && tb->w == w && tb->tab[T_NW]) return QSLC_OK;
    for (auto *&p : tb->tab) {
        if (p) cudaFree(p);
        p = nullptr;
    }
    const unsigned n = s->n;
    const int keys[5][2] = {{int(n) - 1, int(w) - 1}, {int(n) - 2, int(w) - 1},
                            {int(n) - 2, int(w) - 2}, {int(n) - 1, int(w)}, {int(n), int(w)}};
    for (int i = 0; i < 5; i++) {
        tb->len[i] = 0;
        if (keys[i][0] < 0 || keys[i][1] < 0 || keys[i][1] > keys[i][0]) continue;
        const uint64_t cnt = np_choose(unsigned(keys[i][0]), unsigned(keys[i][1]));
        tb->len[i] = cnt;
        if (cnt == 0) continue;
        if (cudaMalloc(&tb->tab[i], cnt * 4) != cudaSuccess) {
            cudaGetLastError();
            return fail(QSLC_EOOM, "out of device memory for NP lookup tables");
        }
        k_np_build_table<<<grid_for(cnt), 256, 0, s->stream>>>(tb->tab[i], cnt, unsigned(keys[i][0]),
                                                               unsigned(keys[i][1]));
        s->launches++;
        QSLC_CUDA(cudaGetLastError());
    }
    tb->n = n;
    tb->w = w;
    return QSLC_OK;
}

template <class T>
static int np_gate_t(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle)
{
    NPTables *tb = tables_of(s);
    auto *st = static_cast<cplx<T> *>(s->amps);
    const uint32_t *rt = d_rank_tab;
    const unsigned w = s->nones;
    cudaStream_t str = s->stream;
    const T a = T(angle);
    auto single = [&](auto kind_tag, int ti, unsigned t1, unsigned t2, uint32_t add, Coef<T> k) {
        constexpr int KIND = decltype(kind_tag)::value;
        const uint64_t cnt = tb->len[ti];
        if (cnt == 0) return;
        const unsigned pat = sizeof(T) == 8 ? pattern_for(k, pattern_np_diag()) : 0u;
        auto go = [&](auto c) {
            k_np_single<T, KIND, decltype(c)::value><<<grid_for(cnt), 256, 0, str>>>(st, tb->tab[ti], cnt, rt,
                                                                                     t1, t2, add, k, pat);
        };
        if constexpr (KIND == NP_NEG1 || KIND == NP_CZ)
            go(std::integral_constant<unsigned, 0u>{});
        else
            with_pattern<QSLC_NP_DIAG_PATTERNS>(pat, go);
        s->launches++;
    };
    auto pair = [&](auto kind_tag, Coef<T> k) {
        constexpr int KIND = decltype(kind_tag)::value;
        const uint64_t cnt = tb->len[T_N2W1];
        if (cnt == 0) return;
        const unsigned lo = q1 < q2 ? q1 : q2, hi = q1 < q2 ? q2 : q1;
        uint32_t b1 = 1u << q1, b2 = 1u << q2;
        if (KIND == NP_SWAP) { b1 = 1u << lo; b2 = 1u << hi; }   // :259-260
        const unsigned pat = sizeof(T) != 8 ? 0u : (KIND == NP_H ? pattern_h() : pattern_for(k, pattern_np_pair()));
        auto go = [&](auto c) {
            k_np_pair<T, KIND, decltype(c)::value><<<grid_for(cnt), 256, 0, str>>>(
                st, tb->tab[T_N2W1], cnt, rt, lo, hi, b1, b2, k, pat);
        };
        if constexpr (KIND == NP_SWAP)
            go(std::integral_constant<unsigned, 0u>{});
        else if constexpr (KIND == NP_H)
            with_pattern<QSLC_H_PATTERNS>(pat, go);
        else
            with_pattern<QSLC_NP_PAIR_PATTERNS>(pat, go);
        s->launches++;
    };
    const unsigned lo = q1 < q2 ? q1 : q2, hi = q1 < q2 ? q2 : q1;
    const uint32_t both = (1u << q1) | (1u << q2);
    switch (gate) {
    case QSLC_PHASE:       // np/gates.cpp:33-57
        single(std::integral_constant<int, NP_PHASE1>{}, T_N1W1, q1, 0, 1u << q1,
               coef<T>(T(std::cos(a)), T(std::sin(a))));
        break;
    case QSLC_PAULI_Z:     // :59-80
        single(std::integral_constant<int, NP_NEG1>{}, T_N1W1, q1, 0, 1u << q1, Coef<T>{});
        break;
    case QSLC_ROTATE_Z: {  // :83-113: e^{-ia/2} on |0>, then phase(a/2)
        single(std::integral_constant<int, NP_RZ0>{}, T_N1W, q1, 0, 0u,
               coef<T>(T(std::cos(a / 2)), T(std::sin(a / 2))));
        const T h = a / 2;
        single(std::integral_constant<int, NP_PHASE1>{}, T_N1W1, q1, 0, 1u << q1,
               coef<T>(T(std::cos(h)), T(std::sin(h))));
        break;
    }
    case QSLC_CONTROL_Z:   // :118-151
        if (w >= 2)
            single(std::integral_constant<int, NP_CZ>{}, T_N2W2, lo, hi, both, Coef<T>{});
        break;
    case QSLC_CONTROL_PHASE:   // :195-233
        if (w >= 2)
            single(std::integral_constant<int, NP_CPHASE>{}, T_N2W2, lo, hi, both,
                   coef<T>(T(std::cos(a)), T(std::sin(a))));
        break;
    case QSLC_CONTROL_ROTATE_Z: {  // :154-192, q1 = control
        single(std::integral_constant<int, NP_CRZ01>{}, T_N2W1, lo, hi, 1u << q1,
               coef<T>(T(std::cos(a / 2)), T(std::sin(a / 2))));
        const T h = a / 2;
        if (w >= 2)
            single(std::integral_constant<int, NP_CPHASE>{}, T_N2W2, lo, hi, both,
                   coef<T>(T(std::cos(h)), T(std::sin(h))));
        break;
    }
    case QSLC_SWAP:
        pair(std::integral_constant<int, NP_SWAP>{}, Coef<T>{});
        break;
    case QSLC_FSWAP:       // :267-275: swap, then controlZ
        pair(std::integral_constant<int, NP_SWAP>{}, Coef<T>{});
        if (w >= 2)
            single(std::integral_constant<int, NP_CZ>{}, T_N2W2, lo, hi, both, Coef<T>{});
        break;
    case QSLC_NP_ROTATE_X:
        pair(std::integral_constant<int, NP_RX>{}, coef<T>(T(std::cos(a / 2)), T(std::sin(a / 2))));
        break;
    case QSLC_NP_ROTATE_Y:
        pair(std::integral_constant<int, NP_RY>{}, coef<T>(T(std::cos(a / 2)), T(std::sin(a / 2))));
        break;
    case QSLC_NP_HADAMARD:
        pair(std::integral_constant<int, NP_H>{}, sqrt2_coef<T>());
        break;
    default:
        return fail(QSLC_EINVAL, "gate " + std::to_string(gate) +
                                     " is not one of the number-preserving gates");
    }
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

int np_gate(qslc_state *s, int gate, unsigned q1, unsigned q2, double angle)
{
    return s->dtype == QSLC_C128 ? np_gate_t<double>(s, gate, q1, q2, angle)
                                 : np_gate_t<float>(s, gate, q1, q2, angle);
}

template <class T>
static int np_collapse_t(qslc_state *s, unsigned t, unsigned o, double factor)
{
    NPTables *tb = tables_of(s);
    auto *st = static_cast<cplx<T> *>(s->amps);
    const int keep = o ? T_N1W1 : T_N1W, drop = o ? T_N1W : T_N1W1;
    if (tb->len[keep]) {
        k_np_scale<T><<<grid_for(tb->len[keep]), 256, 0, s->stream>>>(
            st, tb->tab[keep], tb->len[keep], d_rank_tab, t, o, T(factor), 0);
        s->launches++;
    }
    if (tb->len[drop]) {
        k_np_scale<T><<<grid_for(tb->len[drop]), 256, 0, s->stream>>>(
            st, tb->tab[drop], tb->len[drop], d_rank_tab, t, o ^ 1u, T(0), 1);
        s->launches++;
    }
    QSLC_CUDA(cudaGetLastError());
    return QSLC_OK;
}

int np_collapse(qslc_state *s, unsigned targ, unsigned outcome, double factor)
{
    return s->dtype == QSLC_C128 ? np_collapse_t<double>(s, targ, outcome, factor)
                                 : np_collapse_t<float>(s, targ, outcome, factor);
}

template <class T>
static int np_prob_t(qslc_state *s, unsigned t, unsigned o, double *out)
{
    NPTables *tb = tables_of(s);
    ProdNPMask<T> pr{static_cast<const cplx<T> *>(s->amps), tb->tab[T_NW], t, o};
    SeqOut<T> so;
    int rc = seq_run<ProdNPMask<T>, T, T>(s, pr, s->namps, false, so);
    if (rc) return rc;
    *out = double(so.total);
    return QSLC_OK;
}

int np_prob(qslc_state *s, unsigned targ, unsigned outcome, double *out)
{
    return s->dtype == QSLC_C128 ? np_prob_t<double>(s, targ, outcome, out)
                                 : np_prob_t<float>(s, targ, outcome, out);
}

// The NP sampling CDF runs in Fp (Dist::prob is Fp, np.hpp:63-66).
template <class T>
static int np_sample_t(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    NPTables *tb = tables_of(s);
    ProdNPAll<T> pr{static_cast<const cplx<T> *>(s->amps), tb->tab[T_NW]};
    const unsigned w = s->nones;
    const unsigned nq = s->n;
    auto host_index = [nq, w](uint64_t j) -> uint64_t { return unrank_of(j, nq, w); };
    return seq_sample<ProdNPAll<T>, T, T>(s, pr, s->namps, u, n, out, host_index);
}

// sampleAll2 over the weight-w sector (np/measure.cpp:259-289)
template <class T>
static int np_sample2_t(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    NPTables *tb = tables_of(s);
    ProdNPAll<T> pr{static_cast<const cplx<T> *>(s->amps), tb->tab[T_NW]};
    const unsigned w = s->nones, nq = s->n;
    auto host_index = [nq, w](uint64_t j) -> uint64_t { return unrank_of(j, nq, w); };
    return seq_sample<ProdNPAll<T>, T, T>(s, pr, s->namps, u, n, out, host_index, true);
}

int np_sample_all2(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    return s->dtype == QSLC_C128 ? np_sample2_t<double>(s, u, n, out)
                                 : np_sample2_t<float>(s, u, n, out);
}

int np_sample_all(qslc_state *s, const double *u, uint64_t n, uint64_t *out)
{
    return s->dtype == QSLC_C128 ? np_sample_t<double>(s, u, n, out)
                                 : np_sample_t<float>(s, u, n, out);
}

// getState: scatter the slots into a full 2^n host vector, zeros elsewhere.
int np_expand(qslc_state *s, void *host_full)
{
    std::vector<unsigned char> comp(s->namps * s->amp_bytes());
    QSLC_CUDA(cudaMemcpyAsync(comp.data(), s->amps, comp.size(), cudaMemcpyDeviceToHost, s->stream));
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    np_scatter(comp.data(), host_full, s->n, s->nones, s->amp_bytes());
    return QSLC_OK;
}

// setState: gather the weight-w amplitudes (w already validated).
int np_compress(qslc_state *s, const void *host_full, unsigned w)
{
    std::vector<unsigned char> comp(choose_u64(s->n, w) * s->amp_bytes());
    np_gather(host_full, comp.data(), s->n, w, s->amp_bytes());
    QSLC_CUDA(cudaMemcpyAsync(s->amps, comp.data(), comp.size(), cudaMemcpyHostToDevice, s->stream));
    QSLC_CUDA(cudaStreamSynchronize(s->stream));
    return QSLC_OK;
}

}  // namespace qslc
