// batch.cu -- the batching form: thousands of small circuits in one
// persistent launch, replayed from a CUDA graph.
//
// Each instance is a hardware-efficient ansatz on n qubits: L layers of
// rotateY on every qubit, rotateZ on every qubit, then controlNot(q, q+1)
// for q = 0..n-2; afterwards prob(q, 0) and prob(q, 1) for every q and a
// sampleAll draw per uniform.  The per-instance result is the one qsl's
// Default backend gives for the same calls (gates.cpp, measure.cpp), bit
// for bit: the gates run in the reference's order with its rounding, the
// probabilities are sequential sums in index order, and the sampling CDF is
// the sequential double sum merged against the instance's sorted uniforms
// (the first index whose running sum reaches a uniform is its outcome, as
// drawSample's search returns, measure.cpp:164-188).
//
// Schedule: one CTA of 1024 threads per resident slot pulls instances,
// largest first, from an atomic counter.  A state of up to SMEM_STATE bytes
// lives in shared memory for its whole circuit and never touches HBM; a
// larger one works in the CTA's slot of a global arena (L2 / HBM).  The
// probabilities use n threads (one sequential sum per qubit) and the CDF
// one more thread, running side by side.
#include "qslc_internal.cuh"
#include "replay.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace qslc {
namespace {

constexpr int BATCH_THREADS = 1024;
constexpr size_t SMEM_STATE = 128 * 1024;

struct InstDesc {
    uint32_t n, L;
    uint64_t coef;      // offset of its coefficients: L*n*4 values (cy, sy, cz, sz)
    uint64_t probs;     // offset of its 2n probabilities
    uint64_t shots;     // offset of its shots (sorted-uniform order)
};

template <class T>
__device__ __forceinline__ void ry_pair(cplx<T> &a0, cplx<T> &a1, T c, T s)
{   // gates.cpp:169-174
    using R = rn<T>;
    cplx<T> r0, r1;
    r0.x = R::sub(R::mul(a0.x, c), R::mul(a1.x, s));
    r0.y = R::sub(R::mul(a0.y, c), R::mul(a1.y, s));
    r1.x = R::add(R::mul(a0.x, s), R::mul(a1.x, c));
    r1.y = R::add(R::mul(a0.y, s), R::mul(a1.y, c));
    a0 = r0;
    a1 = r1;
}

template <class T>
__device__ __forceinline__ void rz_pair(cplx<T> &a0, cplx<T> &a1, T c, T s)
{   // gates.cpp:200-205
    using R = rn<T>;
    cplx<T> r0, r1;
    r0.x = R::add(R::mul(a0.x, c), R::mul(a0.y, s));
    r0.y = R::sub(R::mul(a0.y, c), R::mul(a0.x, s));
    r1.x = R::sub(R::mul(a1.x, c), R::mul(a1.y, s));
    r1.y = R::add(R::mul(a1.y, c), R::mul(a1.x, s));
    a0 = r0;
    a1 = r1;
}

template <class T>
__device__ void run_instance(cplx<T> *st, const InstDesc &d, const T *__restrict__ coef,
                             T *__restrict__ probs, const double *__restrict__ u_sorted,
                             uint64_t *__restrict__ shots, uint32_t nshots)
{
    const uint32_t n = d.n;
    const uint64_t dim = uint64_t(1) << n, half = dim >> 1;
    const unsigned tid = threadIdx.x, nt = blockDim.x;
    for (uint64_t i = tid; i < dim; i += nt) {
        cplx<T> z;
        z.x = T(i == 0 ? 1 : 0);
        z.y = T(0);
        st[i] = z;
    }
    __syncthreads();
    const T *cf = coef + d.coef;
    for (uint32_t l = 0; l < d.L; l++) {
        const T *lc = cf + uint64_t(l) * n * 4;
        for (uint32_t q = 0; q < n; q++) {           // rotateY on every qubit
            const T c = lc[4 * q], s = lc[4 * q + 1];
            const uint64_t bit = uint64_t(1) << q;
            for (uint64_t j = tid; j < half; j += nt) {
                uint64_t i0 = insert0(j, q);
                cplx<T> a0 = st[i0], a1 = st[i0 | bit];
                ry_pair<T>(a0, a1, c, s);
                st[i0] = a0;
                st[i0 | bit] = a1;
            }
            __syncthreads();
        }
        for (uint32_t q = 0; q < n; q++) {           // rotateZ on every qubit
            const T c = lc[4 * q + 2], s = lc[4 * q + 3];
            const uint64_t bit = uint64_t(1) << q;
            for (uint64_t j = tid; j < half; j += nt) {
                uint64_t i0 = insert0(j, q);
                cplx<T> a0 = st[i0], a1 = st[i0 | bit];
                rz_pair<T>(a0, a1, c, s);
                st[i0] = a0;
                st[i0 | bit] = a1;
            }
            __syncthreads();
        }
        for (uint32_t q = 0; q + 1 < n; q++) {       // controlNot(q, q+1), gates.cpp:215-240
            const uint64_t cb = uint64_t(1) << q, tb = uint64_t(1) << (q + 1);
            for (uint64_t j = tid; j < (dim >> 2); j += nt) {
                uint64_t x1 = insert00(j, q, q + 1) | cb;
                cplx<T> a = st[x1], b = st[x1 | tb];
                st[x1] = b;
                st[x1 | tb] = a;
            }
            __syncthreads();
        }
    }
    // prob(q, o): sequential Fp sums in index order (measure.cpp:126-147)
    T *pr = probs + d.probs;
    if (tid < 2 * n) {
        const uint32_t q = tid >> 1, o = tid & 1;
        const uint64_t ob = uint64_t(o) << q;
        T p = T(0);
        for (uint64_t j = 0; j < half; j++) {
            const cplx<T> a = st[insert0(j, q) | ob];
            p = rn<T>::add(p, norm2_rn(a.x, a.y));
        }
        pr[2 * q + o] = p;
    } else if (tid == 2 * n) {
        // sampling: the double running sum over all amplitudes, merged
        // against the sorted uniforms (measure.cpp:60-78, :164-188)
        const double *u = u_sorted;
        uint64_t *out = shots + d.shots;
        uint32_t k = 0;
        double run = 0.0;
        for (uint64_t i = 0; i < dim && k < nshots; i++) {
            const cplx<T> a = st[i];
            const T p = norm2_rn(a.x, a.y);
            run = __dadd_rn(run, double(p));
            while (k < nshots && u[k] <= run) out[k++] = i;
        }
        for (; k < nshots; k++) out[k] = 0;           // above the total: index 0
    }
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(BATCH_THREADS) k_batch(const InstDesc *__restrict__ inst,
                                                         const uint32_t *__restrict__ order,
                                                         uint32_t ninst, unsigned *counter,
                                                         const T *__restrict__ coef,
                                                         T *__restrict__ probs,
                                                         const double *__restrict__ usorted,
                                                         uint64_t *__restrict__ shots,
                                                         uint32_t nshots, cplx<T> *arena,
                                                         uint64_t slot_amps)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t next;
    cplx<T> *sm = reinterpret_cast<cplx<T> *>(smem_raw);
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(counter, 1u);
        __syncthreads();
        const uint32_t w = next;
        __syncthreads();
        if (w >= ninst) break;
        const uint32_t id = order[w];
        const InstDesc d = inst[id];
        const bool on_chip = (uint64_t(1) << d.n) * sizeof(cplx<T>) <= SMEM_STATE;
        cplx<T> *st = on_chip ? sm : arena + uint64_t(blockIdx.x) * slot_amps;
        run_instance<T>(st, d, coef, probs, usorted + uint64_t(id) * nshots, shots, nshots);
    }
}

}  // namespace
}  // namespace qslc

using namespace qslc;

struct qslc_batch {
    int dtype = QSLC_C128;
    uint32_t ninst = 0, nshots = 0;
    std::vector<InstDesc> inst;
    std::vector<uint32_t> order;
    uint64_t ncoef = 0, nprobs = 0, nshot_total = 0;
    cudaStream_t stream = nullptr;
    void *d_inst = nullptr, *d_order = nullptr, *d_counter = nullptr, *d_coef = nullptr;
    void *d_probs = nullptr, *d_u = nullptr, *d_shots = nullptr, *d_arena = nullptr;
    uint64_t slot_amps = 0;
    unsigned grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t runs = 0;
};

namespace {

void batch_free(qslc_batch *b)
{
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : {b->d_inst, b->d_order, b->d_counter, b->d_coef, b->d_probs, b->d_u, b->d_shots,
                    b->d_arena})
        if (p) cudaFree(p);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

template <class T>
int capture(qslc_batch *b)
{
    const size_t smem = SMEM_STATE;
    QSLC_CUDA(cudaFuncSetAttribute(k_batch<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    QSLC_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(b->d_counter, 0, sizeof(unsigned), b->stream);
    k_batch<T><<<b->grid, BATCH_THREADS, smem, b->stream>>>(
        static_cast<const InstDesc *>(b->d_inst), static_cast<const uint32_t *>(b->d_order), b->ninst,
        static_cast<unsigned *>(b->d_counter), static_cast<const T *>(b->d_coef),
        static_cast<T *>(b->d_probs), static_cast<const double *>(b->d_u),
        static_cast<uint64_t *>(b->d_shots), b->nshots, static_cast<cplx<T> *>(b->d_arena), b->slot_amps);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    b->graph = g;
    QSLC_CUDA(cudaGraphInstantiate(&b->exec, g, 0));
    return QSLC_OK;
}

template <class T>
int run_t(qslc_batch *b, const double *angles, const double *u, double *probs, uint64_t *shots)
{
    // coefficients exactly as the reference computes them (gates.cpp:154-155,
    // :185-186): Fp cos/sin of Fp(angle)/2
    std::vector<T> coef(b->ncoef);
    uint64_t a = 0;
    for (uint32_t i = 0; i < b->ninst; i++) {
        const InstDesc &d = b->inst[i];
        for (uint64_t k = 0; k < uint64_t(d.L) * d.n; k++) {
            const T ry = T(angles[a + 2 * k]), rz = T(angles[a + 2 * k + 1]);
            T *c = &coef[d.coef + 4 * k];
            c[0] = T(std::cos(ry / 2));
            c[1] = T(std::sin(ry / 2));
            c[2] = T(std::cos(rz / 2));
            c[3] = T(std::sin(rz / 2));
        }
        a += 2 * uint64_t(d.L) * d.n;
    }
    // sort each instance's uniforms; shots come back in sorted order
    const uint32_t ns = b->nshots;
    std::vector<double> us(uint64_t(b->ninst) * ns);
    std::vector<uint32_t> perm(uint64_t(b->ninst) * ns);
    for (uint32_t i = 0; i < b->ninst; i++) {
        uint32_t *pm = perm.data() + uint64_t(i) * ns;
        const double *ui = u + uint64_t(i) * ns;
        std::iota(pm, pm + ns, 0u);
        std::sort(pm, pm + ns, [&](uint32_t x, uint32_t y) { return ui[x] < ui[y]; });
        for (uint32_t k = 0; k < ns; k++) {
            double v = ui[pm[k]];
            if (b->dtype == QSLC_C64) v = double(float(v));   // the reference draws Fp uniforms
            us[uint64_t(i) * ns + k] = v;
        }
    }
    QSLC_CUDA(cudaMemcpyAsync(b->d_coef, coef.data(), coef.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream));
    QSLC_CUDA(cudaMemcpyAsync(b->d_u, us.data(), us.size() * 8, cudaMemcpyHostToDevice, b->stream));
    QSLC_CUDA(cudaGraphLaunch(b->exec, b->stream));
    std::vector<T> pr(b->nprobs);
    std::vector<uint64_t> sh(b->nshot_total);
    QSLC_CUDA(cudaMemcpyAsync(pr.data(), b->d_probs, pr.size() * sizeof(T), cudaMemcpyDeviceToHost, b->stream));
    QSLC_CUDA(cudaMemcpyAsync(sh.data(), b->d_shots, sh.size() * 8, cudaMemcpyDeviceToHost, b->stream));
    QSLC_CUDA(cudaStreamSynchronize(b->stream));
    QSLC_CUDA(cudaGetLastError());
    for (uint64_t i = 0; i < b->nprobs; i++) probs[i] = double(pr[i]);
    for (uint32_t i = 0; i < b->ninst; i++)
        for (uint32_t k = 0; k < ns; k++)
            shots[uint64_t(i) * ns + perm[uint64_t(i) * ns + k]] = sh[b->inst[i].shots + k];
    b->runs++;
    return QSLC_OK;
}

}  // namespace

extern "C" int qslc_batch_create(int dtype, uint32_t ninst, const uint32_t *nqubits,
                                 const uint32_t *nlayers, uint32_t nshots, qslc_batch **out)
{
    if (!out || !nqubits || !nlayers || ninst == 0) return fail(QSLC_EINVAL, "bad batch arguments");
    *out = nullptr;
    if (dtype != QSLC_C128 && dtype != QSLC_C64) return fail(QSLC_EINVAL, "unknown dtype");
    auto *b = new qslc_batch();
    b->dtype = dtype;
    b->ninst = ninst;
    b->nshots = nshots;
    b->inst.resize(ninst);
    uint32_t nmax = 0;
    for (uint32_t i = 0; i < ninst; i++) {
        if (nqubits[i] < 2 || nqubits[i] > 26) {
            delete b;
            return fail(QSLC_EINVAL, "batch instances take 2..26 qubits");
        }
        InstDesc &d = b->inst[i];
        d.n = nqubits[i];
        d.L = nlayers[i];
        d.coef = b->ncoef;
        d.probs = b->nprobs;
        d.shots = b->nshot_total;
        b->ncoef += uint64_t(d.L) * d.n * 4;
        b->nprobs += 2 * uint64_t(d.n);
        b->nshot_total += nshots;
        nmax = std::max(nmax, d.n);
    }
    // largest instances first, so the long ones start early
    b->order.resize(ninst);
    std::iota(b->order.begin(), b->order.end(), 0u);
    std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t x, uint32_t y) {
        return (uint64_t(b->inst[x].L) << b->inst[x].n) > (uint64_t(b->inst[y].L) << b->inst[y].n);
    });
    const size_t ab = dtype == QSLC_C128 ? 16 : 8, fb = dtype == QSLC_C128 ? 8 : 4;
    b->grid = sm_count();
    b->slot_amps = (uint64_t(1) << nmax) * ab > SMEM_STATE ? (uint64_t(1) << nmax) : 0;
    int rc = QSLC_OK;
    auto alloc = [&](void **p, size_t bytes) {
        if (rc) return;
        if (bytes == 0) bytes = 16;
        if (cudaMalloc(p, bytes) != cudaSuccess) {
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
    alloc(&b->d_arena, size_t(b->grid) * b->slot_amps * ab);
    if (!rc && cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "stream creation failed");
    if (!rc && cudaMemcpy(b->d_inst, b->inst.data(), ninst * sizeof(InstDesc), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "upload failed");
    if (!rc && cudaMemcpy(b->d_order, b->order.data(), ninst * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = fail(QSLC_ECUDA, "upload failed");
    if (!rc) rc = dtype == QSLC_C128 ? capture<double>(b) : capture<float>(b);
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
    if (!b || !angles || !probs || (!uniforms && b->nshots) || (!shots && b->nshots))
        return fail(QSLC_EINVAL, "null pointer");
    return b->dtype == QSLC_C128 ? run_t<double>(b, angles, uniforms, probs, shots)
                                 : run_t<float>(b, angles, uniforms, probs, shots);
}

extern "C" int qslc_batch_destroy(qslc_batch *b)
{
    batch_free(b);
    return QSLC_OK;
}
