// bsa_mlp.cu -- the Mesher's zone-refinement proposer: a small MLP
//   x (din) -> W -> W -> W (ReLU) -> 1 logit,  P(refine) = sigmoid(logit)
// with BF16 weights and FP32 accumulation, trained on the device by its own forward and
// backward kernels: binary cross-entropy (hard or soft targets) with per-sample weights,
// Adam on FP32 master weights, the BF16 copy refreshed after every step.  No counterpart in
// the reference (its Mesher refines by fixed policies); the proposer only chooses which zones
// the plain refinement criterion evaluates at the next lattice level.
//
// Parameter order (flattened, FP32 master / BF16 working copy):
//   W1[W][din] b1[W] W2[W][W] b2[W] W3[W][W] b3[W] w4[W] b4
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"

namespace bsa {
namespace mlp {

constexpr int kMaxNets = 8;

struct Buf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t n) {
        if (n <= bytes && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class T> T *as() const { return (T *)p; }
};

struct Net {
    bool used = false;
    int din = 0, W = 0;
    long long np = 0;  // parameters
    long long step = 0;
    Buf master, wbf, grad, m1, m2;                         // parameters, BF16 copy, gradient, Adam moments
    Buf x, y, sw, z1, z2, z3, logit, d1, d2, d3, dl, red;  // batch data and activations
    int cap = 0;                                           // batch capacity of the activation buffers
    cudaStream_t st = nullptr;
    long long off_b1() const { return (long long)W * din; }
    long long off_W2() const { return off_b1() + W; }
    long long off_b2() const { return off_W2() + (long long)W * W; }
    long long off_W3() const { return off_b2() + W; }
    long long off_b3() const { return off_W3() + (long long)W * W; }
    long long off_w4() const { return off_b3() + W; }
    long long off_b4() const { return off_w4() + W; }
};

Net g_nets[kMaxNets];
std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

// ---------------------------------------------------------------- kernels
// out[b][o] = act(sum_i in[b][i] W[o][i] + bias[o]); W, bias BF16; FP32 accumulation.
// relu != 0: ReLU.  One block per sample, the input row staged in shared memory.
__global__ void k_dense(int n, int nin, int nout, const float *__restrict__ in, const __nv_bfloat16 *__restrict__ Wt,
                        const __nv_bfloat16 *__restrict__ bias, int relu, float *__restrict__ out) {
    __shared__ float row[128];
    const int b = blockIdx.x;
    for (int i = threadIdx.x; i < nin; i += blockDim.x) row[i] = in[(size_t)b * nin + i];
    __syncthreads();
    for (int o = threadIdx.x; o < nout; o += blockDim.x) {
        float s = __bfloat162float(bias[o]);
        const __nv_bfloat16 *w = Wt + (size_t)o * nin;
        for (int i = 0; i < nin; ++i) s = fmaf(row[i], __bfloat162float(w[i]), s);
        out[(size_t)b * nout + o] = relu ? fmaxf(s, 0.f) : s;
    }
}

// Weighted binary cross-entropy on the logits: dl[b] = sw_b (sigmoid(z_b) - y_b) / sum(sw),
// lossv[b] = sw_b * loss_b / sum(sw) (summed on the host).
__global__ void k_bce(int n, const float *__restrict__ z, const float *__restrict__ y, const float *__restrict__ sw,
                      float inv_wsum, float *__restrict__ dl, float *__restrict__ lossv) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const float zz = z[b], p = 1.f / (1.f + expf(-zz));
    // log(1 + exp(-|z|)) + max(z, 0) - y z : the stable form of the cross-entropy
    const float l = log1pf(expf(-fabsf(zz))) + fmaxf(zz, 0.f) - y[b] * zz;
    dl[b] = sw[b] * (p - y[b]) * inv_wsum;
    lossv[b] = sw[b] * l * inv_wsum;
}

// dIn[b][i] = (sum_o dOut[b][o] W[o][i]), zeroed where the input activation is not positive
// (the ReLU derivative; mask = that activation)
__global__ void k_back_act(int n, int nin, int nout, const float *__restrict__ dOut,
                           const __nv_bfloat16 *__restrict__ Wt, const float *__restrict__ mask, float *__restrict__ dIn) {
    __shared__ float drow[128];
    const int b = blockIdx.x;
    for (int o = threadIdx.x; o < nout; o += blockDim.x) drow[o] = dOut[(size_t)b * nout + o];
    __syncthreads();
    for (int i = threadIdx.x; i < nin; i += blockDim.x) {
        float s = 0.f;
        for (int o = 0; o < nout; ++o) s = fmaf(drow[o], __bfloat162float(Wt[(size_t)o * nin + i]), s);
        if (mask && mask[(size_t)b * nin + i] <= 0.f) s = 0.f;
        dIn[(size_t)b * nin + i] = s;
    }
}

// gW[o][i] = sum_b dOut[b][o] in[b][i],  gb[o] = sum_b dOut[b][o]  (fixed order over b)
__global__ void k_back_w(int n, int nin, int nout, const float *__restrict__ dOut, const float *__restrict__ in,
                         float *__restrict__ gW, float *__restrict__ gb) {
    const int o = blockIdx.x;
    for (int i = threadIdx.x; i <= nin; i += blockDim.x) {
        float s = 0.f;
        if (i < nin)
            for (int b = 0; b < n; ++b) s = fmaf(dOut[(size_t)b * nout + o], in[(size_t)b * nin + i], s);
        else
            for (int b = 0; b < n; ++b) s += dOut[(size_t)b * nout + o];
        if (i < nin) gW[(size_t)o * nin + i] = s; else gb[o] = s;
    }
}

__global__ void k_adam(long long np, float lr, float b1, float b2, float eps, float c1, float c2,
                       float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       __nv_bfloat16 *__restrict__ wbf) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    wbf[i] = __float2bfloat16_rn(wi);
}

__global__ void k_to_bf16(long long np, const float *__restrict__ w, __nv_bfloat16 *__restrict__ wbf) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) wbf[i] = __float2bfloat16_rn(w[i]);
}

// ---------------------------------------------------------------- host helpers
cudaError_t ensure_batch(Net &N, int n) {
    if (n <= N.cap) return cudaSuccess;
    cudaError_t e;
    const size_t f = sizeof(float);
    if ((e = N.x.reserve(f * n * N.din)) || (e = N.y.reserve(f * n)) || (e = N.sw.reserve(f * n)) ||
        (e = N.z1.reserve(f * n * N.W)) || (e = N.z2.reserve(f * n * N.W)) || (e = N.z3.reserve(f * n * N.W)) ||
        (e = N.logit.reserve(f * n)) || (e = N.d1.reserve(f * n * N.W)) || (e = N.d2.reserve(f * n * N.W)) ||
        (e = N.d3.reserve(f * n * N.W)) || (e = N.dl.reserve(f * n)) || (e = N.red.reserve(f * n)))
        return e;
    N.cap = n;
    return cudaSuccess;
}

// forward on the n rows at x (device), logits into N.logit
void forward(Net &N, const float *x, int n) {
    const __nv_bfloat16 *w = N.wbf.as<__nv_bfloat16>();
    k_dense<<<n, 128, 0, N.st>>>(n, N.din, N.W, x, w, w + N.off_b1(), 1, N.z1.as<float>());
    k_dense<<<n, 128, 0, N.st>>>(n, N.W, N.W, N.z1.as<float>(), w + N.off_W2(), w + N.off_b2(), 1, N.z2.as<float>());
    k_dense<<<n, 128, 0, N.st>>>(n, N.W, N.W, N.z2.as<float>(), w + N.off_W3(), w + N.off_b3(), 1, N.z3.as<float>());
    k_dense<<<n, 128, 0, N.st>>>(n, N.W, 1, N.z3.as<float>(), w + N.off_w4(), w + N.off_b4(), 0, N.logit.as<float>());
}

// loss + gradient into N.grad for the n rows at x, y, sw (device)
cudaError_t backward(Net &N, const float *x, const float *y, const float *sw, int n, float wsum, float *loss) {
    forward(N, x, n);
    float *g = N.grad.as<float>();
    const __nv_bfloat16 *w = N.wbf.as<__nv_bfloat16>();
    k_bce<<<(n + 255) / 256, 256, 0, N.st>>>(n, N.logit.as<float>(), y, sw, 1.f / wsum, N.dl.as<float>(),
                                             N.red.as<float>());
    // output layer
    k_back_w<<<1, 128, 0, N.st>>>(n, N.W, 1, N.dl.as<float>(), N.z3.as<float>(), g + N.off_w4(), g + N.off_b4());
    k_back_act<<<n, 128, 0, N.st>>>(n, N.W, 1, N.dl.as<float>(), w + N.off_w4(), N.z3.as<float>(), N.d3.as<float>());
    // layer 3
    k_back_w<<<N.W, 128, 0, N.st>>>(n, N.W, N.W, N.d3.as<float>(), N.z2.as<float>(), g + N.off_W3(), g + N.off_b3());
    k_back_act<<<n, 128, 0, N.st>>>(n, N.W, N.W, N.d3.as<float>(), w + N.off_W3(), N.z2.as<float>(), N.d2.as<float>());
    // layer 2
    k_back_w<<<N.W, 128, 0, N.st>>>(n, N.W, N.W, N.d2.as<float>(), N.z1.as<float>(), g + N.off_W2(), g + N.off_b2());
    k_back_act<<<n, 128, 0, N.st>>>(n, N.W, N.W, N.d2.as<float>(), w + N.off_W2(), N.z1.as<float>(), N.d1.as<float>());
    // layer 1
    k_back_w<<<N.W, 128, 0, N.st>>>(n, N.din, N.W, N.d1.as<float>(), x, g, g + N.off_b1());
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    if (loss) {
        std::vector<float> lv(n);
        if ((e = cudaMemcpyAsync(lv.data(), N.red.p, sizeof(float) * n, cudaMemcpyDeviceToHost, N.st)) ||
            (e = cudaStreamSynchronize(N.st)))
            return e;
        double s = 0.0;
        for (float v : lv) s += v;
        *loss = (float)s;
    }
    return cudaSuccess;
}

Net *get(int h) {
    if (h < 0 || h >= kMaxNets || !g_nets[h].used) return nullptr;
    return &g_nets[h];
}

}  // namespace mlp
}  // namespace bsa

using namespace bsa::mlp;

extern "C" {

int bsa_mlp_create(int din, int width, unsigned long long seed) {
    if (din < 1 || din > 128 || width < 1 || width > 128) return fail(BSA_ERR_ARG, "0 < din, width <= 128");
    int h = -1;
    for (int k = 0; k < kMaxNets; ++k)
        if (!g_nets[k].used) { h = k; break; }
    if (h < 0) return fail(BSA_ERR_STATE, "too many networks");
    Net &N = g_nets[h];
    N = Net();
    N.din = din;
    N.W = width;
    N.np = (long long)width * din + width + 2 * ((long long)width * width + width) + width + 1;
    // He-uniform initialisation from a seeded generator (splitmix64), biases zero
    std::vector<float> p(N.np, 0.f);
    uint64_t s = seed;
    auto rnd = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);  // [0, 1)
    };
    auto fill = [&](long long off, long long cnt, int fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (long long i = 0; i < cnt; ++i) p[off + i] = (float)((2.0 * rnd() - 1.0) * a);
    };
    fill(0, (long long)width * din, din);
    fill(N.off_W2(), (long long)width * width, width);
    fill(N.off_W3(), (long long)width * width, width);
    fill(N.off_w4(), width, width);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&N.st, cudaStreamNonBlocking)) || (e = N.master.reserve(4 * N.np)) ||
        (e = N.wbf.reserve(2 * N.np)) || (e = N.grad.reserve(4 * N.np)) || (e = N.m1.reserve(4 * N.np)) ||
        (e = N.m2.reserve(4 * N.np)))
        return fail(BSA_ERR_CUDA, std::string("MLP allocation: ") + cudaGetErrorString(e));
    if ((e = cudaMemcpyAsync(N.master.p, p.data(), 4 * N.np, cudaMemcpyHostToDevice, N.st)) ||
        (e = cudaMemsetAsync(N.m1.p, 0, 4 * N.np, N.st)) || (e = cudaMemsetAsync(N.m2.p, 0, 4 * N.np, N.st)))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    k_to_bf16<<<(unsigned)((N.np + 255) / 256), 256, 0, N.st>>>(N.np, N.master.as<float>(), N.wbf.as<__nv_bfloat16>());
    if ((e = cudaStreamSynchronize(N.st))) return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    N.used = true;
    return h;
}

int bsa_mlp_destroy(int h) {
    Net *N = get(h);
    if (!N) return BSA_ERR_ARG;
    for (Buf *b : {&N->master, &N->wbf, &N->grad, &N->m1, &N->m2, &N->x, &N->y, &N->sw, &N->z1, &N->z2, &N->z3,
                   &N->logit, &N->d1, &N->d2, &N->d3, &N->dl, &N->red})
        b->release();
    if (N->st) cudaStreamDestroy(N->st);
    *N = Net();
    return BSA_OK;
}

long long bsa_mlp_num_params(int h) {
    Net *N = get(h);
    return N ? N->np : BSA_ERR_ARG;
}

// params: FP32 master weights (bf16 == 0) or the BF16 working copy as floats (bf16 != 0)
int bsa_mlp_get_params(int h, float *params, int bf16) {
    Net *N = get(h);
    if (!N || !params) return BSA_ERR_ARG;
    cudaError_t e;
    if (!bf16) {
        if ((e = cudaMemcpyAsync(params, N->master.p, 4 * N->np, cudaMemcpyDeviceToHost, N->st)) ||
            (e = cudaStreamSynchronize(N->st)))
            return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
        return BSA_OK;
    }
    std::vector<__nv_bfloat16> b(N->np);
    if ((e = cudaMemcpyAsync(b.data(), N->wbf.p, 2 * N->np, cudaMemcpyDeviceToHost, N->st)) ||
        (e = cudaStreamSynchronize(N->st)))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    for (long long i = 0; i < N->np; ++i) {
        uint16_t u;
        std::memcpy(&u, &b[i], 2);
        const uint32_t f = (uint32_t)u << 16;
        std::memcpy(&params[i], &f, 4);
    }
    return BSA_OK;
}

int bsa_mlp_set_params(int h, const float *params) {
    Net *N = get(h);
    if (!N || !params) return BSA_ERR_ARG;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(N->master.p, params, 4 * N->np, cudaMemcpyHostToDevice, N->st)))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    k_to_bf16<<<(unsigned)((N->np + 255) / 256), 256, 0, N->st>>>(N->np, N->master.as<float>(),
                                                                  N->wbf.as<__nv_bfloat16>());
    if ((e = cudaStreamSynchronize(N->st))) return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    return BSA_OK;
}

int bsa_mlp_forward(int h, const float *x, int n, float *prob) {
    Net *N = get(h);
    if (!N || !x || !prob || n <= 0) return BSA_ERR_ARG;
    cudaError_t e;
    for (int b0 = 0; b0 < n; b0 += 65536) {
        const int nb = n - b0 < 65536 ? n - b0 : 65536;
        if ((e = ensure_batch(*N, nb)) ||
            (e = cudaMemcpyAsync(N->x.p, x + (size_t)b0 * N->din, 4 * (size_t)nb * N->din, cudaMemcpyHostToDevice,
                                 N->st)))
            return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
        forward(*N, N->x.as<float>(), nb);
        std::vector<float> z(nb);
        if ((e = cudaGetLastError()) ||
            (e = cudaMemcpyAsync(z.data(), N->logit.p, 4 * (size_t)nb, cudaMemcpyDeviceToHost, N->st)) ||
            (e = cudaStreamSynchronize(N->st)))
            return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
        for (int b = 0; b < nb; ++b) prob[b0 + b] = 1.f / (1.f + std::exp(-z[b]));
    }
    return BSA_OK;
}

// Loss and gradient (w.r.t. the BF16 working weights) of the weighted cross-entropy.
int bsa_mlp_gradients(int h, const float *x, const float *y, const float *sw, int n, float *loss, float *grads) {
    Net *N = get(h);
    if (!N || !x || !y || !sw || n <= 0 || n > 65536) return BSA_ERR_ARG;
    double wsum = 0.0;
    for (int b = 0; b < n; ++b) wsum += sw[b];
    if (!(wsum > 0.0)) return fail(BSA_ERR_ARG, "sample weights sum to zero");
    cudaError_t e;
    if ((e = ensure_batch(*N, n)) ||
        (e = cudaMemcpyAsync(N->x.p, x, 4 * (size_t)n * N->din, cudaMemcpyHostToDevice, N->st)) ||
        (e = cudaMemcpyAsync(N->y.p, y, 4 * (size_t)n, cudaMemcpyHostToDevice, N->st)) ||
        (e = cudaMemcpyAsync(N->sw.p, sw, 4 * (size_t)n, cudaMemcpyHostToDevice, N->st)))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    if ((e = backward(*N, N->x.as<float>(), N->y.as<float>(), N->sw.as<float>(), n, (float)wsum, loss)))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    if (grads && ((e = cudaMemcpyAsync(grads, N->grad.p, 4 * N->np, cudaMemcpyDeviceToHost, N->st)) ||
                  (e = cudaStreamSynchronize(N->st))))
        return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    return BSA_OK;
}

// Minibatch Adam over the n samples, `epochs` passes in a seeded order.
int bsa_mlp_train(int h, const float *x, const float *y, const float *sw, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float *loss_out) {
    Net *N = get(h);
    if (!N || !x || !y || !sw || n <= 0 || epochs < 1 || batch < 1 || batch > 65536) return BSA_ERR_ARG;
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    uint64_t s = seed ? seed : 0x2545F4914F6CDD1Dull;
    auto nxt = [&]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    };
    std::vector<float> bx((size_t)batch * N->din), by(batch), bw(batch);
    cudaError_t e;
    if ((e = ensure_batch(*N, batch))) return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    float last = 0.f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = n - 1; i > 0; --i) std::swap(idx[i], idx[(int)(nxt() % (uint64_t)(i + 1))]);
        double eloss = 0.0;
        int nb_total = 0;
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nb = n - b0 < batch ? n - b0 : batch;
            double wsum = 0.0;
            for (int b = 0; b < nb; ++b) {
                const int r = idx[b0 + b];
                std::memcpy(&bx[(size_t)b * N->din], x + (size_t)r * N->din, 4 * N->din);
                by[b] = y[r];
                bw[b] = sw[r];
                wsum += sw[r];
            }
            if (!(wsum > 0.0)) continue;
            if ((e = cudaMemcpyAsync(N->x.p, bx.data(), 4 * (size_t)nb * N->din, cudaMemcpyHostToDevice, N->st)) ||
                (e = cudaMemcpyAsync(N->y.p, by.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, N->st)) ||
                (e = cudaMemcpyAsync(N->sw.p, bw.data(), 4 * (size_t)nb, cudaMemcpyHostToDevice, N->st)))
                return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
            float l = 0.f;
            if ((e = backward(*N, N->x.as<float>(), N->y.as<float>(), N->sw.as<float>(), nb, (float)wsum, &l)))
                return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
            ++N->step;
            const float b1 = 0.9f, b2 = 0.999f;
            const float c1 = 1.f / (1.f - std::pow(b1, (float)N->step)), c2 = 1.f / (1.f - std::pow(b2, (float)N->step));
            k_adam<<<(unsigned)((N->np + 255) / 256), 256, 0, N->st>>>(N->np, lr, b1, b2, 1e-8f, c1, c2,
                                                                      N->master.as<float>(), N->grad.as<float>(),
                                                                      N->m1.as<float>(), N->m2.as<float>(),
                                                                      N->wbf.as<__nv_bfloat16>());
            if ((e = cudaGetLastError())) return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
            eloss += l;
            ++nb_total;
        }
        last = nb_total ? (float)(eloss / nb_total) : 0.f;
    }
    if ((e = cudaStreamSynchronize(N->st))) return fail(BSA_ERR_CUDA, cudaGetErrorString(e));
    if (loss_out) *loss_out = last;
    return BSA_OK;
}

const char *bsa_mlp_lastError(void) { return g_err.c_str(); }

}  // extern "C"
