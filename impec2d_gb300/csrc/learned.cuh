// Declarations shared by the tensor-core kernels (learned.cu) and the network built on them
// (learned_net.cu).
#pragma once
#include <cuda_bf16.h>

#include "internal.cuh"

namespace impec {

struct ConvArgs {
    const __nv_bfloat16* X;  // input activations [B][H][W][cin]
    const __nv_bfloat16* W;  // weights [cout_rows][Kp]
    const float* bias;       // [cout] or null
    __nv_bfloat16* Z;        // pre-activation output or null
    __nv_bfloat16* Y;        // output (activation, or gradient) or null
    float* Yf;               // fp32 output or null
    const __nv_bfloat16* skip;  // added after the activation, or null
    const __nv_bfloat16* add;   // gradient mode: added before the gelu' factor, or null
    const __nv_bfloat16* gz;    // gradient mode: pre-activation of the layer whose gradient this is
    __nv_bfloat16* R;           // gradient mode: the raw gradient (acc) as well, or null
    int B, H, W_, cin, cout, Kp, tapsign, act;
    int* err;
};

// Launches k_conv3x3 with the output-channel tile that fits cout.
impec_status launch_conv(const ConvArgs& a, cudaStream_t s);
// Weight gradient dW [cout][conv_kp(cin)] += from dZ [P][cout] and the layer input X [P][cin].
impec_status launch_wgrad(const __nv_bfloat16* dZ, const __nv_bfloat16* X, int B, int H, int W_, int cin, int cout,
                          float* dW, int* err, int num_sms, cudaStream_t s);
int conv_kp(int cin);  // 9 cin rounded up to 64
// Wd [cin][conv_kp(cout)] for the input-gradient convolution of weights W [cout][conv_kp(cin)].
void launch_wt_transpose(const __nv_bfloat16* W, int cin, int cout, __nv_bfloat16* Wd, cudaStream_t s);
int* device_error_flag();
impec_status check_err(int* err, cudaStream_t s, const char* what);

}  // namespace impec
