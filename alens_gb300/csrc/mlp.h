// mlp.h - the learned warm start: a 12 -> 64 -> 64 -> 1 SiLU network that
// predicts each collision constraint's BBPGD multiplier from local pair
// geometry and the previous step's multiplier.  BF16 weights and
// activations on the tensor cores (tcgen05, FP32 accumulation in tensor
// memory), FP32 master weights and Adam.  Used only as the initial iterate
// of BBPGD, so the solve still has to reach the residual tolerance.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

namespace alens {

constexpr int kMlpIn = 12;      // features per constraint
constexpr int kMlpInPad = 16;   // padded to one K = 16 MMA slice
constexpr int kMlpHid = 64;
// FP32 master parameter layout: W1[64][12], b1[64], W2[64][64], b2[64],
// w3[64], b3 (weights stored [out][in])
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHid * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpHid;
constexpr int kOffB2 = kOffW2 + kMlpHid * kMlpHid;
constexpr int kOffW3 = kOffB2 + kMlpHid;
constexpr int kOffB3 = kOffW3 + kMlpHid;
constexpr int kMlpParams = kOffB3 + 1;  // 5057

constexpr int kMlpTile = 128;           // rows per MMA tile (M = 128)
constexpr int kW1Bytes = kMlpHid * kMlpInPad * 2;
constexpr int kW2Bytes = kMlpHid * kMlpHid * 2;

// Device view of a model (by value into kernels).
struct MlpView {
    const float *p;        // FP32 master parameters
    const uint8_t *w1c;    // BF16 W1 (64 x 16, zero-padded), core-matrix layout
    const uint8_t *w2c;    // BF16 W2 (64 x 64)
    const uint8_t *w2tc;   // BF16 W2^T
    const float *w3r;      // w3 rounded to BF16, as FP32
    int *err;              // error flags (bounded waits)
};

struct DevState;

// launchers (kernels_mlp.cu)
void launch_mlp_warm(const DevState &S, const MlpView &V, cudaStream_t st);
void launch_mlp_features(const DevState &S, cudaStream_t st);
void launch_mlp_append(const DevState &S, int k0, int n, float *dsFeat, float *dsLabel, cudaStream_t st);
void launch_mlp_predict(const MlpView &V, const float *feat, int n, float *out, cudaStream_t st);
cudaError_t launch_mlp_train(const MlpView &V, const float *feat, const float *label, long long nData,
                             long long permA, long long permB, long long start, int count, float *grad,
                             double *lossAcc, cudaStream_t st);
void launch_mlp_adam(float *p, const float *grad, float *m, float *v, uint8_t *w1c, uint8_t *w2c,
                     uint8_t *w2tc, float *w3r, float lr, float bc1, float bc2, cudaStream_t st);
void launch_mlp_pack(const float *p, uint8_t *w1c, uint8_t *w2c, uint8_t *w2tc, float *w3r, cudaStream_t st);

// Host object behind AlensMlp.
class MlpModel {
  public:
    MlpModel(unsigned long long seed, long long datasetCap);
    ~MlpModel();
    MlpModel(const MlpModel &) = delete;
    MlpModel &operator=(const MlpModel &) = delete;

    void getParams(float *out);
    void setParams(const float *in);
    long long datasetSize() const { return dsSize_; }
    long long datasetCap() const { return dsCap_; }
    void clearDataset() { dsSize_ = 0; }
    // appends rows to the dataset (device copy on `st`); returns rows added
    long long reserve(long long n) {
        const long long add = n < dsCap_ - dsSize_ ? n : dsCap_ - dsSize_;
        return add > 0 ? add : 0;
    }
    float *dsFeatAt(long long row) { return dsFeat_ + row * kMlpIn; }
    float *dsLabelAt(long long row) { return dsLabel_ + row; }
    void commitRows(long long n) { dsSize_ += n; }
    void uploadDataset(const float *feat, const float *label, long long n);
    void train(int epochs, int batch, float lr, unsigned long long seed, float *lossPerEpoch);
    void gradient(int n, const float *feat, const float *target, float *grad, float *loss);
    void predict(int n, const float *feat, float *out);
    MlpView view() const;
    long long adamSteps() const { return adamStep_; }
    int errFlags();

  private:
    void ensureTemp(long long n);
    void release();
    cudaStream_t stream_ = nullptr;
    float *p_ = nullptr, *m_ = nullptr, *v_ = nullptr, *g_ = nullptr, *w3r_ = nullptr;
    uint8_t *w1c_ = nullptr, *w2c_ = nullptr, *w2tc_ = nullptr;
    int *err_ = nullptr;
    double *loss_ = nullptr;
    float *dsFeat_ = nullptr, *dsLabel_ = nullptr;
    long long dsSize_ = 0, dsCap_ = 0;
    float *tmpFeat_ = nullptr, *tmpLabel_ = nullptr;
    long long tmpCap_ = 0;
    long long adamStep_ = 0;
};

}  // namespace alens
