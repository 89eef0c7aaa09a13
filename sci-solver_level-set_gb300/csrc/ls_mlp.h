// ls_mlp.h -- the learned warm start's network (see ls_mlp.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace lsgb {
namespace mlp {

// Feature builder: 32 1-ring slots x (dx, dy, dz, phi) / h per vertex.
__global__ void k_features(int nlist, const int* vlist, const int* nlist_dev, const int* adj_off, const int* adj,
                           const float* xyz, int nv, const float* phi, float inv_h, const float* vinv_h,
                           __nv_bfloat16* Xo);

class Net {
 public:
  Net() = default;
  ~Net();
  std::string init(unsigned long long seed);
  static int num_params();
  // master parameters [W1 W2 W3 (128x128 each, [out][in]) | b1 b2 b3 | w4 | b4]
  std::string set_params(const float* host);
  std::string get_params(float* host);
  // host-buffer entry points (features rounded to BF16 on the way in)
  std::string predict(const float* X, int n, float* y);
  std::string gradients(const float* X, const float* t, int n, float* g, float* loss);
  std::string train(const float* X, const float* t, int n, int epochs, int batch, float lr, float* last_loss);
  std::string train_dev_upload(const __nv_bfloat16* X, const float* t, int n, int epochs, int batch, float lr,
                               float* last_loss);
  // device entry points on stream st
  std::string forward_dev(const __nv_bfloat16* X, int n, const int* n_dev, int max_n, float* y,
                          __nv_bfloat16* acts, cudaStream_t st);
  // gradients of the batch into G (its loss also added to *loss_sink when
  // given, on the device)
  std::string backward_dev(const __nv_bfloat16* X, int n, const __nv_bfloat16* acts, const float* y, const float* t,
                           cudaStream_t st, float* loss_sink = nullptr);
  std::string train_device(const __nv_bfloat16* X, const float* t, int n, int epochs, int batch, float lr,
                           __nv_bfloat16* acts, float* y, float* last_loss);
  std::string check_err();
  // training pairs (device buffer owned by the network)
  std::string reserve_pairs(long long cap);
  std::string clear_pairs();
  long long num_pairs();
  std::string append_pairs(const __nv_bfloat16* X, const float* t, const int* n_dev, int max_n, cudaStream_t st,
                           long long* added);
  std::string train_pairs(int epochs, int batch, float lr, unsigned long long seed, float* last_loss);
  // |prediction - target| (units of h) of the pairs [first, first + count)
  std::string eval_pairs(long long first, long long count, float* abs_err);

 private:
  cudaStream_t stream_ = nullptr;
  std::vector<void*> allocs_;
  float *P_ = nullptr, *G_ = nullptr, *M1_ = nullptr, *M2_ = nullptr;
  // BF16 weight tiles in the tensor-core operand layout (forward, transposed)
  __nv_bfloat16 *Wb_ = nullptr, *WTb_ = nullptr;
  float* Gp_ = nullptr;        // per-CTA partial gradients of the backward pass [sms_][NG]
  float* loss_acc_ = nullptr;  // the epoch's summed batch losses (device)
  int sms_ = 1;
  int* err_ = nullptr;
  long long step_ = 0;
  __nv_bfloat16* PX_ = nullptr;
  float* PT_ = nullptr;
  unsigned long long* pair_count_ = nullptr;
  long long pair_cap_ = 0;
};

}  // namespace mlp
}  // namespace lsgb
