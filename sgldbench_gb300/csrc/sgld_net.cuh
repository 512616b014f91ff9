// Internal interface of the learned warm start: the 3D convolutional U-Net
// (kernels_net.cu) and its host-side driver (sgld_net.cu).  Nothing here
// crosses the C ABI.
//
// Network (levels L <= 4, widths w_0..w_{L-1}, on a node grid and its
// ceil-halved coarsenings):
//   encoder, level l:  Ea_l = relu(conv3(in_l)),  E_l = relu(conv3(Ea_l)),
//                      in_0 = X,  in_{l+1} = avgpool2(E_l)
//   decoder, level l = L-2 .. 0:
//                      Du_l = relu(conv3(prev))      (on level l+1, w_{l+1} -> w_l)
//                      S_l  = up2(Du_l) + E_l,  D_l = relu(conv3(S_l)),  prev = D_l
//                      (prev starts as E_{L-1})
//   head:              Y = conv1(D_0)  (linear, FP32)
// Parameters, in this order per convolution: W[taps][cin][cout], b[cout];
// convolutions in the order a_0, b_0, .., a_{L-1}, b_{L-1}, u_{L-2}, m_{L-2},
// .., u_0, m_0, head.
#pragma once
#include <cuda_bf16.h>

#include <string>
#include <vector>

#include "sgld_internal.cuh"

namespace sgld {

using bf16 = __nv_bfloat16;
constexpr int NET_MAXL = 4;

struct NetConv {
    int cin, cout, taps, level;
    int64_t w, b;   // offsets into the parameter vector
};

struct NetAct {
    int level = 0, C = 0;
    bf16 *a = nullptr;    // activation [V][C]
    float *g = nullptr;   // dLoss/d(pre-activation) [V][C] (the ReLU mask applied)
};

struct Net {
    int L = 0, cin = 0, cout = 0, width[NET_MAXL] = {};
    int dims[NET_MAXL][3] = {};   // (ny, nx, nz) nodes per level
    int64_t V[NET_MAXL] = {};
    std::vector<NetConv> conv;
    int64_t nparam = 0;
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr, *wpart = nullptr;
    bf16 *wb = nullptr, *wt = nullptr;
    bf16 *wimg = nullptr;   // one convolution's weights as tensor-core operand images (all taps)
    int *tc_err = nullptr;  // set by a tensor-core convolution whose MMA wait gave up
    NetAct X, Ea[NET_MAXL], E[NET_MAXL], P[NET_MAXL], Du[NET_MAXL], S[NET_MAXL], D[NET_MAXL];
    bf16 *x_own = nullptr;   // the network's own input buffer (X.a may point elsewhere)
    float *Y = nullptr, *gY = nullptr, *T = nullptr, *M = nullptr;
    double *mse_part = nullptr, *d_loss = nullptr;
    int step = 0;
    cudaStream_t s = nullptr;
    std::vector<void *> allocs;
};

int net_init(Net &n, int ny, int nx, int nz, int cin, int cout, int L, const int *widths, unsigned long long seed,
             cudaStream_t s, std::string &err);
void net_free(Net &n);
void net_forward(Net &n);                                        // n.X.a -> n.Y
void net_loss(Net &n, const float *T, const float *M);           // n.Y -> n.gY, *n.d_loss
void net_backward(Net &n);                                       // n.gY -> n.g
void net_adam_step(Net &n, float lr);                            // n.g -> n.w, n.wb
// after the work queued on n.s: true when a tensor-core convolution's bounded
// MMA wait gave up (its output is then invalid); clears the flag
bool net_take_error(Net &n);

// kernels_net.cu
void net_init_attributes();
// wimg: scratch for the weight images of the tensor-core path (taps x pad16(cin) x
// pad16(cout) BF16); err: device flag of that path
void net_conv_fwd(const bf16 *in, int cin, const bf16 *w, const float *b, int cout, int taps, int ny, int nx, int nz,
                  bool relu_bf16_out, void *out, bf16 *wimg, int *err, cudaStream_t s);
void net_conv_bwd_data(const float *gout, int cout, const bf16 *w, bf16 *wt, int cin, int taps, int ny, int nx,
                       int nz, const bf16 *mask, float *gin, bool accumulate, bf16 *wimg, int *err, cudaStream_t s);
// kernels_net_tc.cu: the same convolutions on the tensor cores (tcgen05)
bool net_conv_tc_fits(int cin, int cout);
bool net_wgrad_tc_fits(int cin, int cout);
void net_conv_wgrad_tc(const bf16 *in, int cin, const float *gout, int cout, int taps, int ny, int nx, int nz, int S,
                       int64_t vchunk, float *part, float *bpart, int *err, cudaStream_t s);
void net_tc_init_attributes();
void net_conv_fwd_tc(const bf16 *in, int cin, const bf16 *w, const float *b, int cout, int taps, int ny, int nx,
                     int nz, bool relu_bf16_out, void *out, bf16 *wimg, int *err, cudaStream_t s);
void net_conv_bwd_data_tc(const float *gout, int cout, const bf16 *wt, int cin, int taps, int ny, int nx, int nz,
                          const bf16 *mask, float *gin, bool accumulate, bf16 *wimg, int *err, cudaStream_t s);
int net_wgrad_splits(int64_t V);
void net_conv_wgrad(const bf16 *in, int cin, const float *gout, int cout, int taps, int ny, int nx, int nz,
                    float *part, float *gw, float *gb, int *err, cudaStream_t s);
void net_pool(const bf16 *f, int C, const int fd[3], const int cd[3], bf16 *c, cudaStream_t s);
void net_pool_bwd(const float *gc, int C, const int fd[3], const int cd[3], const bf16 *maskf, float *gf,
                  bool accumulate, cudaStream_t s);
void net_up_add(const bf16 *c, const bf16 *skip, int C, const int fd[3], const int cd[3], bf16 *out,
                cudaStream_t s);
void net_up_add_bwd(const float *gs, int C, const int fd[3], const int cd[3], const bf16 *maskc, float *gc,
                    const bf16 *maskskip, float *gskip, bool acc_skip, cudaStream_t s);
int net_mse_blocks(int64_t V);
void net_mse(const float *y, const float *t, const float *m, int C, int64_t V, float *gy, double *part,
             double *loss, cudaStream_t s);
void net_adam(float *w, float *m, float *v, const float *g, bf16 *wb, int64_t n, float lr, float b1, float b2,
              float eps, float c1, float c2, cudaStream_t s);
void net_to_bf16(const float *a, bf16 *b, int64_t n, cudaStream_t s);

}  // namespace sgld

namespace sgld {
// bridge kernels between level vectors and the network (kernels_net.cu)
void net_inject(const double *fine, const int fnodes[3], int S, const int cnodes[3], double *out, cudaStream_t s);
void net_logE(const double *E, const int felems[3], int S, const int cnodes[3], double E0, float *fe,
              cudaStream_t s);
void net_pack(const double *rc, const double *dc, const float *fe, const uint8_t *nflag, int64_t Vc, double sr,
              double sd, bf16 *X, cudaStream_t s);
void net_target(const double *ec, const uint8_t *nflag, int64_t Vc, double se, float *T, float *M, cudaStream_t s);
void net_unpack(const float *Y, const uint8_t *nflag, int64_t Vc, double *out, cudaStream_t s);
void net_axpby(double *y, const double *x, double a, double b, int64_t n, cudaStream_t s);   // y = a x + b y
}  // namespace sgld
