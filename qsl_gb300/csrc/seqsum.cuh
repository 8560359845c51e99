// seqsum.cuh -- bit-exact sequential sums and CDF sampling over a state.
//
// A "producer" describes the sequence the reference sums: element j of
// the sequence is |a|^2 of one stored amplitude, and index(j) is the basis
// index it stands for.  prob(targ, outcome) sums the amplitudes whose bit
// `targ` equals `outcome` in ascending index order (measure.cpp:126-147);
// the sampling CDF sums every amplitude in ascending order
// (measure.cpp:60-78).
//
// The sum is computed in three device passes over tiles of SEQ_TILE
// consecutive elements plus a host walk over per-tile metadata:
//   1. k_seq_tile_sum: an estimate of each tile's sum;
//   2. the host turns the estimates into a guess of the binade the running
//      sum occupies in each tile; k_seq_tile_steps counts, per tile, the
//      grid steps of that binade (replay.cuh) and flags ties;
//   3. the host walks the tiles in order, advancing the exact running sum by
//      u_e * D for every tile whose guess holds and replaying the others
//      term by term (their terms fetched with k_seq_fetch);
//   4. for sampling, k_seq_resolve rebuilds the exact partial sums inside
//      each tile that received a shot and finds, for each uniform u, the
//      first element with partial sum >= u: the reference's binary search
//      over its Dist vector (measure.cpp:164-188) returns the same element.
#pragma once

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <utility>
#include <vector>

#include "qslc_internal.cuh"
#include "replay.cuh"

namespace qslc {

constexpr int SEQ_TILE = 4096;
constexpr int SEQ_TPB = 256;
constexpr int SEQ_PER = SEQ_TILE / SEQ_TPB;
constexpr int SEQ_FETCH_CAP = 256;   // tiles fetched per batch for host replay

// ---------------------------------------------------------------------------
// Producers over the plain 2^n layout.
// ---------------------------------------------------------------------------
template <class T>
struct ProdHalf {        // amplitudes with bit t == outcome, ascending
    const cplx<T> *amps;
    unsigned t;
    uint64_t obit;
    __device__ __forceinline__ uint64_t index(uint64_t j) const { return insert0(j, t) | obit; }
    __device__ __forceinline__ T p(uint64_t j) const
    {
        cplx<T> a = amps[index(j)];
        return norm2_rn(a.x, a.y);
    }
};

template <class T>
struct ProdAll {         // every amplitude, ascending
    const cplx<T> *amps;
    __device__ __forceinline__ uint64_t index(uint64_t j) const { return j; }
    __device__ __forceinline__ T p(uint64_t j) const
    {
        cplx<T> a = amps[j];
        return norm2_rn(a.x, a.y);
    }
};

// ---------------------------------------------------------------------------
// Kernels.  Element j of tile b is b*SEQ_TILE + k*SEQ_TPB + threadIdx.x for
// k = 0..SEQ_PER-1, so every load instruction of a warp is coalesced.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum_d(double v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint64_t warp_sum_u(uint64_t v)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class Prod>
__global__ void __launch_bounds__(SEQ_TPB) k_seq_tile_sum(Prod pr, uint64_t count, uint64_t ntiles,
                                                          double *__restrict__ out)
{
    __shared__ double red[SEQ_TPB / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t b = blockIdx.x; b < ntiles; b += gridDim.x) {
        double acc = 0;
        const uint64_t base = b * SEQ_TILE;
#pragma unroll 4
        for (int k = 0; k < SEQ_PER; k++) {
            uint64_t j = base + uint64_t(k) * SEQ_TPB + threadIdx.x;
            if (j < count) acc += double(pr.p(j));
        }
        acc = warp_sum_d(acc);
        if (lane == 0) red[warp] = acc;
        __syncthreads();
        if (warp == 0) {
            double v = lane < SEQ_TPB / 32 ? red[lane] : 0.0;
            v = warp_sum_d(v);
            if (lane == 0) out[b] = v;
        }
        __syncthreads();
    }
}

// Packs a term's grid steps with its tie bit (bit 63); steps never reach
// 2^62 without also raising `big`.
constexpr uint64_t TIE_BIT = uint64_t(1) << 63;

__device__ __forceinline__ Tx warp_compose(Tx x)
{
    // ordered reduction: after the loop lane 0 holds lane 0 then 1 then ... 31
    const int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        Tx y;
        y.d[0] = __shfl_down_sync(0xffffffffu, x.d[0], off);
        y.d[1] = __shfl_down_sync(0xffffffffu, x.d[1], off);
        if ((lane & (2 * off - 1)) == 0) x = tx_then(x, y);
    }
    return x;
}

__device__ __forceinline__ Tx warp_scan_incl(Tx x)
{
    // inclusive ordered scan: lane l holds lanes 0..l composed in order
    const int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        Tx y;
        y.d[0] = __shfl_up_sync(0xffffffffu, x.d[0], off);
        y.d[1] = __shfl_up_sync(0xffffffffu, x.d[1], off);
        if (lane >= off) x = tx_then(y, x);
    }
    return x;
}

// Grid steps of every term of a tile into `sm` (coalesced loads), and the
// OR of the `big` flags.
template <class Prod, class A>
__device__ __forceinline__ unsigned tile_terms(const Prod &pr, uint64_t count, uint64_t base, int e,
                                               uint64_t *sm)
{
    unsigned big_any = 0;
#pragma unroll 4
    for (int k = 0; k < SEQ_PER; k++) {
        const int i = k * SEQ_TPB + threadIdx.x;
        const uint64_t j = base + uint64_t(i);
        uint64_t v = 0;
        if (j < count) {
            bool tie, big;
            v = grid_steps<A>(A(pr.p(j)), e, tie, big);
            if (big) {
                big_any = 1;
                v = 0;
            }
            if (tie) v |= TIE_BIT;
        }
        sm[i] = v;
    }
    return big_any;
}

// The transducer of this thread's SEQ_PER consecutive terms of `sm`.
__device__ __forceinline__ Tx segment_tx(const uint64_t *sm)
{
    Tx t = tx_identity();
#pragma unroll
    for (int k = 0; k < SEQ_PER; k++) {
        const uint64_t v = sm[threadIdx.x * SEQ_PER + k];
        t = tx_then(t, tx_term(v & ~TIE_BIT, (v & TIE_BIT) != 0));
    }
    return t;
}

template <class Prod, class A>
__global__ void __launch_bounds__(SEQ_TPB) k_seq_tile_steps(Prod pr, uint64_t count, uint64_t ntiles,
                                                            const int16_t *__restrict__ guess,
                                                            uint64_t *__restrict__ steps,
                                                            uint8_t *__restrict__ flags)
{
    __shared__ uint64_t sm[SEQ_TILE];
    __shared__ Tx wtx[SEQ_TPB / 32];
    __shared__ unsigned big_all;
    constexpr uint64_t CAP = uint64_t(1) << (fp_traits<A>::MANT + 1);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t b = blockIdx.x; b < ntiles; b += gridDim.x) {
        if (threadIdx.x == 0) big_all = 0;
        __syncthreads();
        const unsigned big = tile_terms<Prod, A>(pr, count, b * SEQ_TILE, guess[b], sm);
        if (big) atomicOr(&big_all, 1u);
        __syncthreads();
        Tx t = segment_tx(sm);
        // a run of 4096 terms below CAP each stays below 2^62: no overflow
        t = warp_compose(t);
        if (lane == 0) wtx[warp] = t;
        __syncthreads();
        if (threadIdx.x == 0) {
            Tx tot = wtx[0];
            for (int w = 1; w < SEQ_TPB / 32; w++) tot = tx_then(tot, wtx[w]);
            unsigned fl = big_all ? 2u : 0u;
            if (tot.d[0] >= CAP || tot.d[1] >= CAP) fl |= 2u;
            steps[2 * b] = tot.d[0] < CAP ? tot.d[0] : CAP;
            steps[2 * b + 1] = tot.d[1] < CAP ? tot.d[1] : CAP;
            flags[b] = uint8_t(fl);
        }
        __syncthreads();
    }
}

template <class Prod, class P>
__global__ void __launch_bounds__(SEQ_TPB) k_seq_fetch(Prod pr, uint64_t count,
                                                       const uint64_t *__restrict__ tiles, int ntl,
                                                       P *__restrict__ out)
{
    for (int q = blockIdx.x; q < ntl; q += gridDim.x) {
        const uint64_t base = tiles[q] * SEQ_TILE;
        for (int i = threadIdx.x; i < SEQ_TILE; i += SEQ_TPB) {
            uint64_t j = base + i;
            out[uint64_t(q) * SEQ_TILE + i] = j < count ? pr.p(j) : P(0);
        }
    }
}

struct ResolveItem {
    uint64_t tile;
    double start;       // exact running sum before the tile's first element
    int32_t binade;     // binade the sum stays in throughout the tile
    uint32_t shot0;     // first shot (index into the sorted uniforms)
    uint32_t nshot;
    uint32_t strict;    // 1: first partial sum > u (sampleAll2); 0: >= u (sampleAll)
};

template <class Prod, class A>
__global__ void __launch_bounds__(SEQ_TPB) k_seq_resolve(Prod pr, uint64_t count,
                                                         const ResolveItem *__restrict__ items,
                                                         int nitems,
                                                         const double *__restrict__ u_sorted,
                                                         uint64_t *__restrict__ out_sorted)
{
    __shared__ uint64_t pre[SEQ_TILE];
    __shared__ Tx wtx[SEQ_TPB / 32];
    constexpr int MANT = fp_traits<A>::MANT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = blockIdx.x; q < nitems; q += gridDim.x) {
        const ResolveItem it = items[q];
        const uint64_t base = it.tile * SEQ_TILE;
        tile_terms<Prod, A>(pr, count, base, it.binade, pre);
        __syncthreads();
        // running sum before the tile, in grid steps of the tile's binade
        const uint64_t s0 = uint64_t(ldexp(it.start, MANT - it.binade));
        const Tx seg = segment_tx(pre);
        Tx incl = warp_scan_incl(seg);
        if (lane == 31) wtx[warp] = incl;
        __syncthreads();
        Tx before = tx_identity();                 // warps before this one
        for (int w = 0; w < warp; w++) before = tx_then(before, wtx[w]);
        Tx excl_in_warp;
        excl_in_warp.d[0] = __shfl_up_sync(0xffffffffu, incl.d[0], 1);
        excl_in_warp.d[1] = __shfl_up_sync(0xffffffffu, incl.d[1], 1);
        if (lane == 0) excl_in_warp = tx_identity();
        const Tx prefix = tx_then(before, excl_in_warp);
        const uint64_t off = prefix.d[s0 & 1];
        uint64_t loc[SEQ_PER];
        uint64_t run = off;
#pragma unroll
        for (int k = 0; k < SEQ_PER; k++) {
            const uint64_t v = pre[threadIdx.x * SEQ_PER + k];
            const Tx t = tx_term(v & ~TIE_BIT, (v & TIE_BIT) != 0);
            run += t.d[(s0 + run) & 1];
            loc[k] = run;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SEQ_PER; k++) pre[threadIdx.x * SEQ_PER + k] = loc[k];
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < it.nshot; k += SEQ_TPB) {
            const double u = u_sorted[it.shot0 + k];
            int lo = 0, hi = SEQ_TILE - 1;   // first i with partial(i) >= u
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                double v = double(A(ldexp(double(s0 + pre[mid]), it.binade - MANT)));
                if (it.strict ? (v > u) : (v >= u)) hi = mid;
                else lo = mid + 1;
            }
            const uint64_t last = count - 1 - base;   // the tile's last valid element
            out_sorted[it.shot0 + k] = pr.index(base + (uint64_t(lo) < last ? uint64_t(lo) : last));
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Host sequencer.
// ---------------------------------------------------------------------------
template <class A>
struct SeqOut {
    A total = A(0);
    std::vector<A> starts;                                  // per tile
    std::vector<int16_t> guess;
    std::unordered_map<uint64_t, std::vector<A>> partials;  // replayed tiles
    uint64_t replayed = 0;
};

// Device working storage for one sequence of `ntiles` tiles, carved from
// one block; `fetch_cap` tiles of terms can be staged for host replay.
struct SeqScratch {
    double *tile_sum;
    int16_t *guess;
    uint64_t *steps;
    uint8_t *flags;
    uint64_t *fetch_ids;
    void *fetch_buf;
    size_t bytes;
    static size_t align(size_t x) { return (x + 255) & ~size_t(255); }
    static SeqScratch carve(void *base, uint64_t ntiles, size_t p_bytes, int fetch_cap)
    {
        SeqScratch s{};
        char *p = static_cast<char *>(base);
        size_t off = 0;
        s.tile_sum = reinterpret_cast<double *>(p + off); off += align(ntiles * 8);
        s.steps = reinterpret_cast<uint64_t *>(p + off); off += align(ntiles * 16);
        s.guess = reinterpret_cast<int16_t *>(p + off); off += align(ntiles * 2);
        s.flags = reinterpret_cast<uint8_t *>(p + off); off += align(ntiles);
        s.fetch_ids = reinterpret_cast<uint64_t *>(p + off); off += align(size_t(fetch_cap) * 8);
        s.fetch_buf = p + off; off += align(size_t(fetch_cap) * SEQ_TILE * p_bytes);
        s.bytes = off;
        return s;
    }
};

// Host working storage of the walk: per-tile metadata and a small cache of
// staged tiles (`cap` slots of SEQ_TILE terms each).
template <class P>
struct SeqHost {
    double *est;
    uint64_t *steps;
    uint8_t *flags;
    int16_t *guess;
    uint8_t *predicted;
    uint64_t *slot_tile;    // cap entries
    uint64_t *batch;        // cap entries
    P *slot_terms;          // cap * SEQ_TILE
    int cap;
};

// Where a sequence runs: stream, launch counter, device and host storage.
template <class P>
struct SeqEnv {
    cudaStream_t stream;
    uint64_t *launches;
    SeqScratch dev;
    SeqHost<P> host;
    int fetch_cap;
};

template <class A>
inline A grid_value(uint64_t steps, int e)
{
    return A(std::ldexp(double(steps), e - fp_traits<A>::MANT));
}

// The exact sequential sum of producer `pr` over `count` elements.
// starts (optional, ntiles entries): the running sum before each tile.
// on_replay (optional): called with (tile, partial sums) for replayed tiles.
template <class Prod, class P, class A, class OnReplay>
int seq_core(SeqEnv<P> &env, const Prod &pr, uint64_t count, A *total, A *starts,
             OnReplay on_replay, uint64_t *replayed)
{
    using T = fp_traits<A>;
    const uint64_t ntiles = (count + SEQ_TILE - 1) / SEQ_TILE;
    SeqScratch &sc = env.dev;
    SeqHost<P> &h = env.host;
    cudaStream_t str = env.stream;
    const unsigned grid = unsigned(std::min<uint64_t>(ntiles, uint64_t(sm_count()) * 8));

    // pass 1: estimates of the tile sums
    k_seq_tile_sum<Prod><<<grid, SEQ_TPB, 0, str>>>(pr, count, ntiles, sc.tile_sum);
    (*env.launches)++;
    QSLC_CUDA(cudaGetLastError());
    QSLC_CUDA(cudaMemcpyAsync(h.est, sc.tile_sum, ntiles * 8, cudaMemcpyDeviceToHost, str));
    QSLC_CUDA(cudaStreamSynchronize(str));

    // guesses: the binade of the estimated running sum at each tile start
    {
        double run = 0;
        for (uint64_t b = 0; b < ntiles; b++) {
            const double end = run + h.est[b];
            h.guess[b] = int16_t(T::EMIN - 1);
            h.predicted[b] = 0;
            if (h.est[b] != 0) {
                int g0 = binade<A>(A(run)), g1 = binade<A>(A(end));
                h.guess[b] = int16_t(run > 0 ? g0 : g1);
                // near or across a power of two: expect a replay
                double nxt = std::ldexp(1.0, (run > 0 ? g0 : g1) + 1);
                double margin = (sizeof(A) == 8 ? 1e-9 : 1e-4) * nxt;
                if (run <= 0 || g0 != g1 || end + margin >= nxt || g0 < T::EMIN) h.predicted[b] = 1;
            }
            run = end;
        }
    }
    QSLC_CUDA(cudaMemcpyAsync(sc.guess, h.guess, ntiles * 2, cudaMemcpyHostToDevice, str));
    k_seq_tile_steps<Prod, A><<<grid, SEQ_TPB, 0, str>>>(pr, count, ntiles, sc.guess, sc.steps, sc.flags);
    (*env.launches)++;
    QSLC_CUDA(cudaGetLastError());
    QSLC_CUDA(cudaMemcpyAsync(h.steps, sc.steps, ntiles * 16, cudaMemcpyDeviceToHost, str));
    QSLC_CUDA(cudaMemcpyAsync(h.flags, sc.flags, ntiles, cudaMemcpyDeviceToHost, str));
    QSLC_CUDA(cudaStreamSynchronize(str));

    // Staged terms for replays: a tile that needs one is fetched together
    // with the next tiles expected to need one, up to `cap` per batch.
    for (int i = 0; i < h.cap; i++) h.slot_tile[i] = ~uint64_t(0);
    auto terms_of = [&](uint64_t b, const P **out) -> int {
        for (int i = 0; i < h.cap; i++)
            if (h.slot_tile[i] == b) {
                *out = h.slot_terms + size_t(i) * SEQ_TILE;
                return QSLC_OK;
            }
        int cnt = 0;
        h.batch[cnt++] = b;
        for (uint64_t c = b + 1; c < ntiles && cnt < h.cap; c++)
            if (h.est[c] != 0 && (h.predicted[c] || h.flags[c])) h.batch[cnt++] = c;
        QSLC_CUDA(cudaMemcpyAsync(sc.fetch_ids, h.batch, size_t(cnt) * 8, cudaMemcpyHostToDevice, str));
        k_seq_fetch<Prod, P><<<unsigned(std::min(cnt, 1024)), SEQ_TPB, 0, str>>>(
            pr, count, sc.fetch_ids, cnt, static_cast<P *>(sc.fetch_buf));
        (*env.launches)++;
        QSLC_CUDA(cudaGetLastError());
        QSLC_CUDA(cudaMemcpyAsync(h.slot_terms, sc.fetch_buf, size_t(cnt) * SEQ_TILE * sizeof(P),
                                  cudaMemcpyDeviceToHost, str));
        QSLC_CUDA(cudaStreamSynchronize(str));
        for (int i = 0; i < h.cap; i++) h.slot_tile[i] = i < cnt ? h.batch[i] : ~uint64_t(0);
        *out = h.slot_terms;
        return QSLC_OK;
    };

    // the walk
    A sum = A(0);
    uint64_t nrep = 0;
    const uint64_t cap = uint64_t(1) << (T::MANT + 1);
    for (uint64_t b = 0; b < ntiles; b++) {
        if (starts) starts[b] = sum;
        if (h.est[b] == 0) continue;            // every term is zero
        const int e = h.guess[b];
        bool ok = h.flags[b] == 0 && sum > A(0) && binade<A>(sum) == e && e >= T::EMIN;
        if (ok) {
            const uint64_t s0 = uint64_t(std::ldexp(double(sum), T::MANT - e));
            const uint64_t d = h.steps[2 * b + (s0 & 1)];   // ties round to even
            ok = s0 + d < cap;
            if (ok) {
                sum = grid_value<A>(s0 + d, e);
                continue;
            }
        }
        // replay term by term, exactly as the reference adds them
        const P *t = nullptr;
        int r = terms_of(b, &t);
        if (r) return r;
        const uint64_t valid = std::min<uint64_t>(SEQ_TILE, count - b * SEQ_TILE);
        const A before = sum;
        for (uint64_t i = 0; i < valid; i++) {
            volatile A next = sum + A(t[i]);
            sum = next;
        }
        on_replay(b, before, t, valid);
        nrep++;
    }
    *total = sum;
    if (replayed) *replayed = nrep;
    return QSLC_OK;
}

// The same over a handle's growable scratch; the host storage is heap.
template <class Prod, class P, class A>
int seq_run(qslc_state *s, const Prod &pr, uint64_t count, bool keep_partials, SeqOut<A> &out)
{
    const uint64_t ntiles = (count + SEQ_TILE - 1) / SEQ_TILE;
    const int cap = SEQ_FETCH_CAP;
    SeqScratch probe = SeqScratch::carve(nullptr, ntiles, sizeof(P), cap);
    int rc = s->scratch.ensure(probe.bytes);
    if (rc) return rc;
    std::vector<double> est(ntiles);
    std::vector<uint64_t> steps(2 * ntiles), slot_tile(cap), batch(cap);
    std::vector<uint8_t> flags(ntiles), predicted(ntiles);
    out.guess.assign(ntiles, 0);
    std::vector<P> slot_terms(size_t(cap) * SEQ_TILE);
    SeqEnv<P> env{s->stream, &s->launches, SeqScratch::carve(s->scratch.ptr, ntiles, sizeof(P), cap),
                  SeqHost<P>{est.data(), steps.data(), flags.data(), out.guess.data(), predicted.data(),
                             slot_tile.data(), batch.data(), slot_terms.data(), cap},
                  cap};
    out.starts.assign(ntiles, A(0));
    out.partials.clear();
    auto on_replay = [&](uint64_t b, A before, const P *t, uint64_t valid) {
        if (!keep_partials) return;
        std::vector<A> part(SEQ_TILE);
        A run = before;
        for (uint64_t i = 0; i < valid; i++) {
            volatile A next = run + A(t[i]);
            run = next;
            part[i] = run;
        }
        for (uint64_t i = valid; i < SEQ_TILE; i++) part[i] = run;
        out.partials.emplace(b, std::move(part));
    };
    return seq_core<Prod, P, A>(env, pr, count, &out.total, out.starts.data(), on_replay, &out.replayed);
}

// Sampling: for each uniform, the element whose partial sum is the first to
// reach it.  `host_index` maps an element to its basis index for shots that
// land in replayed tiles.  Outcomes go to out[0..n) in the order of u.
// strict (sampleAll2, measure.cpp:237-267): the first element whose
// partial sum exceeds u; a uniform at or above the total lands nowhere and
// is reported as ~0.  Otherwise (sampleAll): the first partial sum >= u,
// and 0 above the total.
template <class Prod, class P, class A, class HostIndex>
int seq_sample(qslc_state *s, const Prod &pr, uint64_t count, const double *u, uint64_t n,
               uint64_t *out, HostIndex host_index, bool strict = false)
{
    SeqOut<A> so;
    int rc = seq_run<Prod, P, A>(s, pr, count, true, so);
    if (rc) return rc;
    const uint64_t ntiles = so.starts.size();
    std::vector<uint32_t> order(n);
    for (uint64_t i = 0; i < n; i++) order[i] = uint32_t(i);
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return u[a] < u[b]; });
    std::vector<double> us(n);
    for (uint64_t i = 0; i < n; i++) us[i] = u[order[i]];

    std::vector<ResolveItem> items;
    std::vector<uint64_t> res(n, 0);
    std::vector<char> on_device(n, 0);
    uint64_t b = 0;
    for (uint64_t k = 0; k < n;) {
        const double uk = us[k];
        const uint64_t none = strict ? ~uint64_t(0) : 0;
        auto reaches = [strict](double v, double x) { return strict ? v > x : v >= x; };
        if (!reaches(double(so.total), uk)) {   // past the total (:167, :258)
            res[k++] = none;
            continue;
        }
        // first tile whose end reaches uk
        while (b < ntiles) {
            double end = (b + 1 < ntiles) ? double(so.starts[b + 1]) : double(so.total);
            if (reaches(end, uk)) break;
            b++;
        }
        if (b >= ntiles) { res[k++] = none; continue; }
        const double end = (b + 1 < ntiles) ? double(so.starts[b + 1]) : double(so.total);
        uint64_t k1 = k;
        while (k1 < n && reaches(end, us[k1])) k1++;
        auto pit = so.partials.find(b);
        if (pit != so.partials.end()) {
            const std::vector<A> &part = pit->second;
            for (uint64_t q = k; q < k1; q++) {
                const double x = us[q];
                uint64_t i = uint64_t(std::find_if(part.begin(), part.end(),
                                                   [&](A v) { return reaches(double(v), x); }) -
                                      part.begin());
                if (i >= SEQ_TILE) i = SEQ_TILE - 1;
                res[q] = host_index(b * SEQ_TILE + i);
            }
        } else {
            ResolveItem it{};
            it.tile = b;
            it.start = double(so.starts[b]);
            it.binade = so.guess[b];
            it.shot0 = uint32_t(k);
            it.nshot = uint32_t(k1 - k);
            it.strict = strict ? 1u : 0u;
            items.push_back(it);
            for (uint64_t q = k; q < k1; q++) on_device[q] = 1;
        }
        k = k1;
    }
    if (!items.empty()) {
        const size_t need = SeqScratch::align(n * 8) * 2 + SeqScratch::align(items.size() * sizeof(ResolveItem));
        rc = s->scratch2.ensure(need);
        if (rc) return rc;
        char *p = static_cast<char *>(s->scratch2.ptr);
        double *d_u = reinterpret_cast<double *>(p);
        uint64_t *d_out = reinterpret_cast<uint64_t *>(p + SeqScratch::align(n * 8));
        ResolveItem *d_items = reinterpret_cast<ResolveItem *>(p + 2 * SeqScratch::align(n * 8));
        cudaStream_t str = s->stream;
        QSLC_CUDA(cudaMemcpyAsync(d_u, us.data(), n * 8, cudaMemcpyHostToDevice, str));
        QSLC_CUDA(cudaMemcpyAsync(d_items, items.data(), items.size() * sizeof(ResolveItem),
                                  cudaMemcpyHostToDevice, str));
        const unsigned grid = unsigned(std::min<size_t>(items.size(), size_t(sm_count()) * 4));
        k_seq_resolve<Prod, A><<<grid, SEQ_TPB, 0, str>>>(pr, count, d_items, int(items.size()), d_u, d_out);
        s->launches++;
        QSLC_CUDA(cudaGetLastError());
        std::vector<uint64_t> dev(n);
        QSLC_CUDA(cudaMemcpyAsync(dev.data(), d_out, n * 8, cudaMemcpyDeviceToHost, str));
        QSLC_CUDA(cudaStreamSynchronize(str));
        for (uint64_t q = 0; q < n; q++)
            if (on_device[q]) res[q] = dev[q];
    }
    for (uint64_t q = 0; q < n; q++) out[order[q]] = res[q];
    return QSLC_OK;
}

}  // namespace qslc
