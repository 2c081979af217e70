// Rank predictor for partialACA: a 10 -> 64 -> 64 -> 1 perceptron (FP32,
// ReLU) that maps an admissible block's geometry to the number of ACA
// crosses it needs.  Inference, training (per-sample forward and backward,
// a deterministic split-batch gradient reduction, Adam) are plain CUDA
// kernels; an epoch of training is captured once as a CUDA graph and
// replayed.
//
// Parameter layout (floats): W1[64][10], b1[64], W2[64][64], b2[64], W3[64], b3.
#include "kernels.hpp"

#include <algorithm>
#include <cmath>
#include <random>

namespace htgpu {

namespace {

constexpr int kIn = kMlpIn, kH = kMlpHidden;
constexpr int oW1 = 0, ob1 = oW1 + kH * kIn, oW2 = ob1 + kH, ob2 = oW2 + kH * kH, oW3 = ob2 + kH, ob3 = oW3 + kH;
static_assert(ob3 + 1 == kMlpParams, "parameter layout");
constexpr int kSplit = 64; // sample slices of the gradient reduction

__device__ __forceinline__ void load_params(float *sp, const float *__restrict__ p) {
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x)
        sp[i] = p[i];
    __syncthreads();
}

// forward of one sample with the parameters in shared memory: h1 after ReLU
// in registers; the second hidden layer one unit at a time (stored to H2 when
// given)
__device__ __forceinline__ float forward(const float *sp, const float *__restrict__ x, float (&h1)[kH], float *H2) {
    float xv[kIn];
#pragma unroll
    for (int k = 0; k < kIn; k++)
        xv[k] = x[k];
#pragma unroll
    for (int i = 0; i < kH; i++) {
        float a = sp[ob1 + i];
#pragma unroll
        for (int k = 0; k < kIn; k++)
            a = fmaf(sp[oW1 + i * kIn + k], xv[k], a);
        h1[i] = fmaxf(a, 0.f);
    }
    float out = sp[ob3];
#pragma unroll 2
    for (int j = 0; j < kH; j++) {
        float a = sp[ob2 + j];
#pragma unroll
        for (int i = 0; i < kH; i++)
            a = fmaf(sp[oW2 + j * kH + i], h1[i], a);
        const float h = fmaxf(a, 0.f);
        if (H2)
            H2[j] = h;
        out = fmaf(sp[oW3 + j], h, out);
    }
    return out;
}

__global__ void __launch_bounds__(128) mlp_predict_kernel(const float *__restrict__ params, const float *__restrict__ X, int n, float *__restrict__ y) {
    __shared__ float sp[kMlpParams];
    load_params(sp, params);
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n)
        return;
    float h1[kH];
    y[b] = forward(sp, X + (size_t)b * kIn, h1, nullptr);
}

// per sample: forward, squared error, backward to the hidden layers;
// loss = mean over the n samples of (out - y)^2
__global__ void __launch_bounds__(128) mlp_sample_kernel(const float *__restrict__ params, const float *__restrict__ X, const float *__restrict__ Y, int n, float *__restrict__ H1,
                                                         float *__restrict__ H2, float *__restrict__ D1, float *__restrict__ D2, float *__restrict__ Dout, float *__restrict__ sq) {
    __shared__ float sp[kMlpParams];
    load_params(sp, params);
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n)
        return;
    float h1[kH];
    float *h2row     = H2 + (size_t)b * kH;
    const float out  = forward(sp, X + (size_t)b * kIn, h1, h2row);
    const float e    = out - Y[b];
    const float dout = 2.f * e / (float)n;
    sq[b]            = e * e;
    Dout[b]          = dout;
    float g1[kH];
#pragma unroll
    for (int i = 0; i < kH; i++)
        g1[i] = 0.f;
#pragma unroll 2
    for (int j = 0; j < kH; j++) {
        const float d2 = h2row[j] > 0.f ? dout * sp[oW3 + j] : 0.f;
        D2[(size_t)b * kH + j] = d2;
#pragma unroll
        for (int i = 0; i < kH; i++)
            g1[i] = fmaf(d2, sp[oW2 + j * kH + i], g1[i]);
    }
#pragma unroll
    for (int i = 0; i < kH; i++) {
        H1[(size_t)b * kH + i] = h1[i];
        D1[(size_t)b * kH + i] = h1[i] > 0.f ? g1[i] : 0.f;
    }
}

// partial gradients over sample slice blockIdx.y: one parameter per thread
__global__ void mlp_grad_kernel(const float *__restrict__ X, int n, const float *__restrict__ H1, const float *__restrict__ H2, const float *__restrict__ D1, const float *__restrict__ D2,
                                const float *__restrict__ Dout, float *__restrict__ part) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams)
        return;
    const int per = (n + kSplit - 1) / kSplit;
    const int b0 = blockIdx.y * per, b1 = min(n, b0 + per);
    float g = 0.f;
    if (p < ob1) {
        const int i = (p - oW1) / kIn, k = (p - oW1) % kIn;
        for (int b = b0; b < b1; b++)
            g = fmaf(D1[(size_t)b * kH + i], X[(size_t)b * kIn + k], g);
    } else if (p < oW2) {
        for (int b = b0; b < b1; b++)
            g += D1[(size_t)b * kH + (p - ob1)];
    } else if (p < ob2) {
        const int j = (p - oW2) / kH, i = (p - oW2) % kH;
        for (int b = b0; b < b1; b++)
            g = fmaf(D2[(size_t)b * kH + j], H1[(size_t)b * kH + i], g);
    } else if (p < oW3) {
        for (int b = b0; b < b1; b++)
            g += D2[(size_t)b * kH + (p - ob2)];
    } else if (p < ob3) {
        for (int b = b0; b < b1; b++)
            g = fmaf(Dout[b], H2[(size_t)b * kH + (p - oW3)], g);
    } else {
        for (int b = b0; b < b1; b++)
            g += Dout[b];
    }
    part[(size_t)blockIdx.y * kMlpParams + p] = g;
}

// slices summed in order; Adam step (t = step number from 1) unless lr == 0
__global__ void mlp_adam_kernel(const float *__restrict__ part, float *__restrict__ params, float *__restrict__ m, float *__restrict__ v, float *__restrict__ grad, const int *__restrict__ step,
                                float lr, float beta1, float beta2, float eps) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kMlpParams)
        return;
    float g = 0.f;
    for (int s = 0; s < kSplit; s++)
        g += part[(size_t)s * kMlpParams + p];
    grad[p] = g;
    if (lr == 0.f)
        return;
    const int t   = *step;
    const float a = beta1 * m[p] + (1.f - beta1) * g;
    const float c = beta2 * v[p] + (1.f - beta2) * g * g;
    m[p]          = a;
    v[p]          = c;
    const float mh = a / (1.f - powf(beta1, (float)t));
    const float vh = c / (1.f - powf(beta2, (float)t));
    params[p] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void mlp_count_kernel(int *step) { ++*step; }

__global__ void mlp_loss_kernel(const float *__restrict__ sq, int n, float *__restrict__ loss) {
    __shared__ float red[256];
    float s = 0.f;
    for (int b = threadIdx.x; b < n; b += blockDim.x)
        s += sq[b];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        *loss = red[0] / (float)n;
}

} // namespace

Mlp::Mlp(unsigned long long seed, int device) : device_(device) {
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    // Glorot-uniform weights, zero biases (seeded)
    std::vector<float> p(kMlpParams, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_in, int fan_out, int count) {
        const float a = std::sqrt(6.f / (float)(fan_in + fan_out));
        std::uniform_real_distribution<float> u(-a, a);
        for (int i = 0; i < count; i++)
            p[off + i] = u(rng);
    };
    fill(oW1, kIn, kH, kH * kIn);
    fill(oW2, kH, kH, kH * kH);
    fill(oW3, kH, 1, kH);
    p[ob3] = 0.f;
    params_.upload(p, stream_);
    m_.alloc(kMlpParams);
    v_.alloc(kMlpParams);
    grad_.alloc(kMlpParams);
    part_.alloc((size_t)kSplit * kMlpParams);
    step_.alloc(1);
    loss_.alloc(1);
    HTGPU_CUDA(cudaMemsetAsync(m_.p, 0, sizeof(float) * kMlpParams, stream_));
    HTGPU_CUDA(cudaMemsetAsync(v_.p, 0, sizeof(float) * kMlpParams, stream_));
    HTGPU_CUDA(cudaMemsetAsync(step_.p, 0, sizeof(int), stream_));
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

Mlp::~Mlp() {
    if (graph_exec_)
        cudaGraphExecDestroy(graph_exec_);
    if (stream_)
        cudaStreamDestroy(stream_);
}

void Mlp::set_params(const float *p) {
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaMemcpyAsync(params_.p, p, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, stream_));
    HTGPU_CUDA(cudaMemsetAsync(m_.p, 0, sizeof(float) * kMlpParams, stream_));
    HTGPU_CUDA(cudaMemsetAsync(v_.p, 0, sizeof(float) * kMlpParams, stream_));
    HTGPU_CUDA(cudaMemsetAsync(step_.p, 0, sizeof(int), stream_));
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Mlp::get_params(float *p) {
    HTGPU_CUDA(cudaSetDevice(device_));
    HTGPU_CUDA(cudaMemcpyAsync(p, params_.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream_));
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

void Mlp::ensure_batch(int n) {
    if (n <= batch_cap_)
        return;
    // a captured epoch refers to the old buffers: it must not be replayed
    if (graph_exec_) {
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    h1_.alloc((size_t)n * kH);
    h2_.alloc((size_t)n * kH);
    d1_.alloc((size_t)n * kH);
    d2_.alloc((size_t)n * kH);
    dout_.alloc(n);
    sq_.alloc(n);
    batch_cap_ = n;
}

// one forward/backward/reduction (and Adam update when lr > 0) over the n
// samples at X, Y (device pointers), on stream st
void Mlp::step_launches(const float *X, const float *Y, int n, float lr, cudaStream_t st) {
    mlp_sample_kernel<<<(n + 127) / 128, 128, 0, st>>>(params_.p, X, Y, n, h1_.p, h2_.p, d1_.p, d2_.p, dout_.p, sq_.p);
    mlp_grad_kernel<<<dim3((kMlpParams + 127) / 128, kSplit), 128, 0, st>>>(X, n, h1_.p, h2_.p, d1_.p, d2_.p, dout_.p, part_.p);
    if (lr > 0.f)
        mlp_count_kernel<<<1, 1, 0, st>>>(step_.p);
    mlp_adam_kernel<<<(kMlpParams + 127) / 128, 128, 0, st>>>(part_.p, params_.p, m_.p, v_.p, grad_.p, step_.p, lr, 0.9f, 0.999f, 1e-8f);
    HTGPU_CUDA(cudaGetLastError());
}

float Mlp::gradient(const float *X, const float *Y, int n, float *grad) {
    require(n > 0, "no samples");
    HTGPU_CUDA(cudaSetDevice(device_));
    DevBuf<float> dx, dy;
    dx.upload(X, (size_t)n * kIn, stream_);
    dy.upload(Y, (size_t)n, stream_);
    ensure_batch(n);
    step_launches(dx.p, dy.p, n, 0.f, stream_);
    mlp_loss_kernel<<<1, 256, 0, stream_>>>(sq_.p, n, loss_.p);
    HTGPU_CUDA(cudaGetLastError());
    float loss = 0.f;
    HTGPU_CUDA(cudaMemcpyAsync(grad, grad_.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream_));
    HTGPU_CUDA(cudaMemcpyAsync(&loss, loss_.p, sizeof(float), cudaMemcpyDeviceToHost, stream_));
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
    return loss;
}

void Mlp::train(const float *X, const float *Y, int n, int epochs, int batch, float lr, unsigned long long seed, float *loss_per_epoch) {
    require(n > 0 && epochs > 0 && batch > 0 && lr > 0.f, "training needs samples, epochs, a batch size and a learning rate");
    HTGPU_CUDA(cudaSetDevice(device_));
    batch             = std::min(batch, n);
    const int nbatch  = n / batch; // full batches; the shuffled remainder waits for the next epoch
    DevBuf<float> dx, dy;
    dx.alloc((size_t)n * kIn);
    dy.alloc((size_t)n);
    // every buffer the epoch graph or the loss pass touches is sized here,
    // before the capture: nothing is reallocated while the graph exists
    ensure_batch(std::max(n, batch));
    // an epoch = nbatch steps over consecutive slices of the (reshuffled)
    // device copy of the samples: captured once, replayed every epoch
    if (graph_exec_) {
        cudaGraphExecDestroy(graph_exec_);
        graph_exec_ = nullptr;
    }
    cudaGraph_t graph;
    HTGPU_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < nbatch; s++)
        step_launches(dx.p + (size_t)s * batch * kIn, dy.p + (size_t)s * batch, batch, lr, stream_);
    HTGPU_CUDA(cudaStreamEndCapture(stream_, &graph));
    HTGPU_CUDA(cudaGraphInstantiate(&graph_exec_, graph, 0));
    cudaGraphDestroy(graph);

    std::vector<int> order(n);
    std::vector<float> xs((size_t)n * kIn), ys(n);
    std::mt19937_64 rng(seed);
    for (int i = 0; i < n; i++)
        order[i] = i;
    DevBuf<float> all_x, all_y;
    all_x.upload(X, (size_t)n * kIn, stream_);
    all_y.upload(Y, (size_t)n, stream_);
    for (int e = 0; e < epochs; e++) {
        std::shuffle(order.begin(), order.end(), rng);
        for (int i = 0; i < n; i++) {
            for (int k = 0; k < kIn; k++)
                xs[(size_t)i * kIn + k] = X[(size_t)order[i] * kIn + k];
            ys[i] = Y[order[i]];
        }
        HTGPU_CUDA(cudaMemcpyAsync(dx.p, xs.data(), sizeof(float) * xs.size(), cudaMemcpyHostToDevice, stream_));
        HTGPU_CUDA(cudaMemcpyAsync(dy.p, ys.data(), sizeof(float) * ys.size(), cudaMemcpyHostToDevice, stream_));
        HTGPU_CUDA(cudaGraphLaunch(graph_exec_, stream_));
        if (loss_per_epoch) {
            // loss over all samples with the parameters after this epoch
            mlp_sample_kernel<<<(n + 127) / 128, 128, 0, stream_>>>(params_.p, all_x.p, all_y.p, n, h1_.p, h2_.p, d1_.p, d2_.p, dout_.p, sq_.p);
            mlp_loss_kernel<<<1, 256, 0, stream_>>>(sq_.p, n, loss_.p);
            HTGPU_CUDA(cudaGetLastError());
            HTGPU_CUDA(cudaMemcpyAsync(loss_per_epoch + e, loss_.p, sizeof(float), cudaMemcpyDeviceToHost, stream_));
        }
        HTGPU_CUDA(cudaStreamSynchronize(stream_)); // xs / ys are refilled next epoch
    }
    // the graph reads dx / dy, which end with this call
    cudaGraphExecDestroy(graph_exec_);
    graph_exec_ = nullptr;
}

void Mlp::predict_device(const float *X, int n, float *y, cudaStream_t st) {
    if (n <= 0)
        return;
    mlp_predict_kernel<<<(n + 127) / 128, 128, 0, st>>>(params_.p, X, n, y);
    HTGPU_CUDA(cudaGetLastError());
}

void Mlp::predict(const float *X, int n, float *y) {
    HTGPU_CUDA(cudaSetDevice(device_));
    if (n <= 0)
        return;
    DevBuf<float> dx, dy;
    dx.upload(X, (size_t)n * kIn, stream_);
    dy.alloc(n);
    predict_device(dx.p, n, dy.p, stream_);
    HTGPU_CUDA(cudaMemcpyAsync(y, dy.p, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
    HTGPU_CUDA(cudaStreamSynchronize(stream_));
}

// the features of an admissible block (all scale-free): log2 sizes, radii
// and separation relative to the centre distance, accuracy and kernel
void block_features(int M, int N, double rad_t, double rad_s, const double *ctr_t, const double *ctr_s, double eps, int kernel_id, float *f) {
    double d2 = 0;
    for (int k = 0; k < 3; k++)
        d2 += (ctr_t[k] - ctr_s[k]) * (ctr_t[k] - ctr_s[k]);
    const double d  = std::max(std::sqrt(d2), 1e-300);
    const double rt = rad_t / d, rs = rad_s / d;
    f[0] = (float)(std::log2((double)M) / 16.0);
    f[1] = (float)(std::log2((double)N) / 16.0);
    f[2] = (float)rt;
    f[3] = (float)rs;
    f[4] = (float)(rt + rs);
    f[5] = (float)(std::log2(std::max(1.0 / std::max(rt + rs, 1e-12), 1e-12)) / 4.0);
    f[6] = (float)(-std::log10(eps) / 6.0);
    f[7] = (float)kernel_id;
    f[8] = (float)(std::log2((double)M * (double)N) / 32.0);
    f[9] = (float)(std::min(rad_t, rad_s) / std::max(std::max(rad_t, rad_s), 1e-300));
}

} // namespace htgpu
