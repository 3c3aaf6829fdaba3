// Host-side state of the learned velocity preconditioner (csrc/unet.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "internal.cuh"

namespace uwg {
namespace unet {

constexpr int kMaxLevels = 6;
constexpr int kInChannels = 8;     // residual (3), V-cycle answer (3), log10 viscosity (1), zero (1)
constexpr int kUsedChannels = 7;   // channels the test hooks exchange with the host

// zero-padded voxel grid of one level (channels-last tensors of nv voxels)
struct Vol {
    int px, py, pz;
    int64_t nv;
};

struct Conv {
    int cin, cout;
    int64_t w_off, b_off;                         // offsets in the parameter vector
    DArray<__nv_bfloat16> w16, wflip;             // [27][cin][cout] and [27][cout][cin] (flipped)
};

struct Net {
    int levels = 0, base = 0;
    int64_t nnx = 0, nny = 0, nnz = 0, nn = 0;    // node grid of the mesh the net was built for
    Vol vol[kMaxLevels];
    int ch[kMaxLevels];                           // channels of level l
    std::vector<Conv> convs;                      // enc(l, k) = 2l + k; dec(l, k) = 2 levels + 2l + k
    int64_t head_w = 0, head_b = 0;
    int64_t nparams = 0;
    DArray<float> params, grads, adam_m, adam_v;
    int adam_t = 0;
    float out_scale = 1.0f;                       // target scale learned from the training set

    // preconditioner state: node log10 viscosity, scratch scalar
    DArray<float> logeta;
    DArray<double> sumsq;
    // training set: inputs (r/rms(r), V(r)/rms(V(r))) [sample][6][nn] and targets
    // (e - V(r))/rms(V(r))/out_scale [sample][3][nn]
    DArray<float> data_x, data_y;
    std::vector<double> ysq;                      // |target|^2 per sample
    int nsamples = 0;
    DArray<unsigned char> modes;                  // random-field mode table

    // activations (BF16, channels-last) and the head output (FP32, [3][nv0])
    DArray<__nv_bfloat16> x0;
    DArray<__nv_bfloat16> enc_a[kMaxLevels], enc_b[kMaxLevels], pool[kMaxLevels];
    DArray<__nv_bfloat16> dec_cat[kMaxLevels], dec_a[kMaxLevels], dec_b[kMaxLevels];
    DArray<float> out;
    // gradients (FP32)
    DArray<float> gout, g_enc_a[kMaxLevels], g_enc_b[kMaxLevels], g_in[kMaxLevels];
    DArray<float> g_dec_a[kMaxLevels], g_dec_b[kMaxLevels], g_cat[kMaxLevels];
    DArray<float> part;                           // per-block partial gradients (ordered sums)
    DArray<uint32_t> tc_err;                      // set by a tensor-core kernel whose MMA wait timed out

    int enc(int l, int k) const { return 2 * l + k; }
    int dec(int l, int k) const { return 2 * levels + 2 * l + k; }
    int cin_of_level(int l) const { return l == 0 ? kInChannels : ch[l - 1]; }
};

// Builds the network for the context's mesh (weights He-uniform from `seed`, head zero).
void create(Context& c, Net& n, int levels, int base, uint64_t seed);
// BF16 copies of the FP32 master weights (after an update or a parameter upload).
void pack(Context& c, Net& n);
// Forward pass on n.x0 -> n.out.
void forward(Context& c, Net& n);
// Backward pass from n.gout (gradient of the head output, [3][nv0]); adds into n.grads.
// n.g_in[0] receives the gradient of the input tensor.
void backward(Context& c, Net& n);
// Input tensor from host node arrays input[7][nn] (test hook); output back to out[3][nn].
void set_input_host(Context& c, Net& n, const float* input);
void get_output_host(Context& c, Net& n, float* output);
// Gradient of the output from host grad[3][nn] (zero on padding voxels); input gradient to host [7][nn].
void set_grad_output_host(Context& c, Net& n, const float* grad);
void get_input_grad_host(Context& c, Net& n, float* grad_input);

// Throws (and clears the flag) when a tensor-core kernel of the network gave up waiting for its
// MMAs; synchronises the stream.
void check_errors(Context& c, Net& n);
// node log10 viscosity from the assembled material points (needed before correct / training)
void prepare_viscosity(Context& c, Net& n);
// z += network correction for residual r, z holding the V-cycle's answer V(r) (node SoA [3][nn])
template <typename T>
void correct(Context& c, Net& n, const T* r, T* z);
// random multi-scale velocity field (0 on fixed dofs) into e[3][nn]
void random_field(Context& c, Net& n, uint64_t seed, double* e);
void dataset_reserve(Context& c, Net& n, int nsamples);
void dataset_add(Context& c, Net& n, const double* r, const double* e, const double* v);
void dataset_finish(Context& c, Net& n);
// Adam on the relative squared error; the last 10% of the samples are held out
void train(Context& c, Net& n, int epochs, int batch, float lr, uint64_t seed, double* train_loss,
           double* holdout_ratio);

}  // namespace unet
}  // namespace uwg
