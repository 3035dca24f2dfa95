// mlp.cu - host side of the learned warm-start model (AlensMlp): device
// parameters, Adam state, the (feature, converged multiplier) dataset and
// the training loop.  Kernels are in kernels_mlp.cu.
#include "mlp.h"

#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine.h"

namespace alens {

#define MCK(call)                                                  \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) throw CudaFailure(e_, #call);       \
    } while (0)

namespace {

unsigned long long splitmix64(unsigned long long &s) {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double uniform01(unsigned long long &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

template <class T>
T *dalloc(size_t n) {
    void *p = nullptr;
    MCK(cudaMalloc(&p, (n > 0 ? n : 1) * sizeof(T)));
    return (T *)p;
}

}  // namespace

MlpModel::MlpModel(unsigned long long seed, long long datasetCap) {
    if (datasetCap < 0 || datasetCap > (1LL << 31)) throw ApiError(ALENS_INVALID_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        throw ApiError(ALENS_NO_DEVICE);
    }
    try {
        MCK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        p_ = dalloc<float>(kMlpParams);
        m_ = dalloc<float>(kMlpParams);
        v_ = dalloc<float>(kMlpParams);
        g_ = dalloc<float>(kMlpParams);
        w3r_ = dalloc<float>(kMlpHid);
        w1c_ = dalloc<uint8_t>(kW1Bytes);
        w2c_ = dalloc<uint8_t>(kW2Bytes);
        w2tc_ = dalloc<uint8_t>(kW2Bytes);
        err_ = dalloc<int>(1);
        loss_ = dalloc<double>(1);
        dsCap_ = datasetCap;
        if (dsCap_ > 0) {
            dsFeat_ = dalloc<float>((size_t)dsCap_ * kMlpIn);
            dsLabel_ = dalloc<float>((size_t)dsCap_);
        }
        MCK(cudaMemset(err_, 0, sizeof(int)));
        MCK(cudaMemset(w1c_, 0, kW1Bytes));
        // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases
        std::vector<float> h(kMlpParams, 0.0f);
        unsigned long long s = seed;
        auto fill = [&](int off, int n, int fanIn) {
            const double a = 1.0 / std::sqrt((double)fanIn);
            for (int i = 0; i < n; i++) h[off + i] = (float)((2.0 * uniform01(s) - 1.0) * a);
        };
        fill(kOffW1, kMlpHid * kMlpIn, kMlpIn);
        fill(kOffW2, kMlpHid * kMlpHid, kMlpHid);
        fill(kOffW3, kMlpHid, kMlpHid);
        setParams(h.data());
    } catch (...) {
        release();
        throw;
    }
}

MlpModel::~MlpModel() { release(); }

void MlpModel::release() {
    if (stream_) cudaStreamSynchronize(stream_);
    for (void *p : {(void *)p_, (void *)m_, (void *)v_, (void *)g_, (void *)w3r_, (void *)w1c_, (void *)w2c_,
                    (void *)w2tc_, (void *)err_, (void *)loss_, (void *)dsFeat_, (void *)dsLabel_,
                    (void *)tmpFeat_, (void *)tmpLabel_})
        if (p) cudaFree(p);
    p_ = m_ = v_ = g_ = w3r_ = nullptr;
    w1c_ = w2c_ = w2tc_ = nullptr;
    err_ = nullptr;
    loss_ = nullptr;
    dsFeat_ = dsLabel_ = tmpFeat_ = tmpLabel_ = nullptr;
    if (stream_) cudaStreamDestroy(stream_);
    stream_ = nullptr;
}

MlpView MlpModel::view() const {
    MlpView V;
    V.p = p_;
    V.w1c = w1c_;
    V.w2c = w2c_;
    V.w2tc = w2tc_;
    V.w3r = w3r_;
    V.err = err_;
    return V;
}

int MlpModel::errFlags() {
    int e = 0;
    MCK(cudaMemcpyAsync(&e, err_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    return e;
}

void MlpModel::getParams(float *out) {
    MCK(cudaMemcpyAsync(out, p_, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
}

void MlpModel::setParams(const float *in) {
    for (int i = 0; i < kMlpParams; i++)
        if (!std::isfinite(in[i])) throw ApiError(ALENS_INVALID_ARG);
    MCK(cudaMemcpyAsync(p_, in, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, stream_));
    MCK(cudaMemsetAsync(m_, 0, sizeof(float) * kMlpParams, stream_));
    MCK(cudaMemsetAsync(v_, 0, sizeof(float) * kMlpParams, stream_));
    launch_mlp_pack(p_, w1c_, w2c_, w2tc_, w3r_, stream_);
    MCK(cudaGetLastError());
    MCK(cudaStreamSynchronize(stream_));
    adamStep_ = 0;
}

void MlpModel::ensureTemp(long long n) {
    if (n <= tmpCap_) return;
    if (tmpFeat_) cudaFree(tmpFeat_);
    if (tmpLabel_) cudaFree(tmpLabel_);
    tmpFeat_ = tmpLabel_ = nullptr;
    tmpCap_ = 0;
    tmpFeat_ = dalloc<float>((size_t)n * kMlpIn);
    tmpLabel_ = dalloc<float>((size_t)n);
    tmpCap_ = n;
}

void MlpModel::uploadDataset(const float *feat, const float *label, long long n) {
    if (n < 0 || (n > 0 && (!feat || !label))) throw ApiError(ALENS_INVALID_ARG);
    const long long add = reserve(n);
    if (add < n) throw ApiError(ALENS_CAPACITY);
    if (add == 0) return;
    MCK(cudaMemcpyAsync(dsFeatAt(dsSize_), feat, sizeof(float) * kMlpIn * add, cudaMemcpyHostToDevice, stream_));
    MCK(cudaMemcpyAsync(dsLabelAt(dsSize_), label, sizeof(float) * add, cudaMemcpyHostToDevice, stream_));
    MCK(cudaStreamSynchronize(stream_));
    commitRows(add);
}

void MlpModel::train(int epochs, int batch, float lr, unsigned long long seed, float *lossPerEpoch) {
    if (epochs < 0 || batch < 1 || !(lr > 0.0f) || dsSize_ < 1) throw ApiError(ALENS_INVALID_ARG);
    const long long N = dsSize_;
    unsigned long long s = seed ^ 0x5DEECE66DULL;
    for (int ep = 0; ep < epochs; ep++) {
        // this epoch's order: i -> (a i + b) mod N with gcd(a, N) = 1
        long long a = 1, b = 0;
        if (N > 1) {
            do {
                a = 1 + (long long)(splitmix64(s) % (unsigned long long)(N - 1));
            } while (std::gcd(a, N) != 1);
            b = (long long)(splitmix64(s) % (unsigned long long)N);
        }
        MCK(cudaMemsetAsync(loss_, 0, sizeof(double), stream_));
        for (long long start = 0; start < N; start += batch) {
            const int count = (int)(N - start < batch ? N - start : batch);
            MCK(cudaMemsetAsync(g_, 0, sizeof(float) * kMlpParams, stream_));
            MCK(launch_mlp_train(view(), dsFeat_, dsLabel_, N, a, b, start, count, g_, loss_, stream_));
            adamStep_++;
            const float bc1 = (float)(1.0 - std::pow(0.9, (double)adamStep_));
            const float bc2 = (float)(1.0 - std::pow(0.999, (double)adamStep_));
            launch_mlp_adam(p_, g_, m_, v_, w1c_, w2c_, w2tc_, w3r_, lr, bc1, bc2, stream_);
            MCK(cudaGetLastError());
        }
        double l = 0.0;
        MCK(cudaMemcpyAsync(&l, loss_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
        MCK(cudaStreamSynchronize(stream_));
        if (errFlags() & kErrTimeout) throw ApiError(ALENS_TIMEOUT);
        if (lossPerEpoch) lossPerEpoch[ep] = (float)(l / (double)N);
    }
}

void MlpModel::gradient(int n, const float *feat, const float *target, float *grad, float *loss) {
    if (n < 1 || !feat || !target || !grad) throw ApiError(ALENS_INVALID_ARG);
    ensureTemp(n);
    MCK(cudaMemcpyAsync(tmpFeat_, feat, sizeof(float) * kMlpIn * (size_t)n, cudaMemcpyHostToDevice, stream_));
    MCK(cudaMemcpyAsync(tmpLabel_, target, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, stream_));
    MCK(cudaMemsetAsync(g_, 0, sizeof(float) * kMlpParams, stream_));
    MCK(cudaMemsetAsync(loss_, 0, sizeof(double), stream_));
    MCK(launch_mlp_train(view(), tmpFeat_, tmpLabel_, n, 1, 0, 0, n, g_, loss_, stream_));
    double l = 0.0;
    MCK(cudaMemcpyAsync(grad, g_, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaMemcpyAsync(&l, loss_, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    if (errFlags() & kErrTimeout) throw ApiError(ALENS_TIMEOUT);
    if (loss) *loss = (float)(l / (double)n);
}

void MlpModel::predict(int n, const float *feat, float *out) {
    if (n < 0 || (n > 0 && (!feat || !out))) throw ApiError(ALENS_INVALID_ARG);
    if (n == 0) return;
    ensureTemp(n);
    MCK(cudaMemcpyAsync(tmpFeat_, feat, sizeof(float) * kMlpIn * (size_t)n, cudaMemcpyHostToDevice, stream_));
    launch_mlp_predict(view(), tmpFeat_, n, tmpLabel_, stream_);
    MCK(cudaGetLastError());
    MCK(cudaMemcpyAsync(out, tmpLabel_, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, stream_));
    MCK(cudaStreamSynchronize(stream_));
    if (errFlags() & kErrTimeout) throw ApiError(ALENS_TIMEOUT);
}

}  // namespace alens
