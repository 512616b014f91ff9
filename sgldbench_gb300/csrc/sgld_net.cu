// Host driver of the learned warm start's U-Net (layout and graph in
// sgld_net.cuh) and its C ABI (include/sgld_gpu.h, sgld_net_*).  Every
// operation is a launch of kernels_net.cu on the network's stream; the host
// only sequences them.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/sgld_gpu.h"
#include "sgld_net.cuh"

namespace sgld {

namespace {

template <typename T>
cudaError_t nalloc(Net &n, T **p, int64_t count) {
    *p = nullptr;
    if (count <= 0) count = 1;
    const cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)count);
    if (e == cudaSuccess) n.allocs.push_back(*p);
    return e;
}

// splitmix64 (Steele, Lea, Flood 2014): the seeded stream of the initial weights
struct SplitMix {
    unsigned long long x;
    unsigned long long next() {
        unsigned long long z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }   // [0, 1)
};

const int *dim3_of(const Net &n, int l) { return n.dims[l]; }

void conv_fwd(Net &n, int k, const bf16 *in, void *out, bool relu) {
    const NetConv &c = n.conv[k];
    const int *d = dim3_of(n, c.level);
    net_conv_fwd(in, c.cin, n.wb + c.w, n.w + c.b, c.cout, c.taps, d[0], d[1], d[2], relu, out, n.wimg, n.tc_err,
                 n.s);
}

// dW, db of convolution k from its input activation and the gradient of its output
void conv_wgrad(Net &n, int k, const bf16 *in, const float *gout) {
    const NetConv &c = n.conv[k];
    const int *d = dim3_of(n, c.level);
    net_conv_wgrad(in, c.cin, gout, c.cout, c.taps, d[0], d[1], d[2], n.wpart, n.g + c.w, n.g + c.b, n.tc_err,
                   n.s);
}

// gradient of convolution k's input: gin (=/+=) mask(conv^T(gout))
void conv_bwd(Net &n, int k, const float *gout, const bf16 *mask, float *gin, bool acc) {
    const NetConv &c = n.conv[k];
    const int *d = dim3_of(n, c.level);
    net_conv_bwd_data(gout, c.cout, n.wb + c.w, n.wt, c.cin, c.taps, d[0], d[1], d[2], mask, gin, acc, n.wimg,
                      n.tc_err, n.s);
}

int conv_a(int l) { return 2 * l; }
int conv_b(int l) { return 2 * l + 1; }
int conv_u(const Net &n, int l) { return 2 * n.L + 2 * (n.L - 2 - l); }
int conv_m(const Net &n, int l) { return 2 * n.L + 2 * (n.L - 2 - l) + 1; }
int conv_head(const Net &n) { return 4 * n.L - 2; }

}  // namespace

int net_init(Net &n, int ny, int nx, int nz, int cin, int cout, int L, const int *widths, unsigned long long seed,
             cudaStream_t s, std::string &err) {
    if (ny < 1 || nx < 1 || nz < 1 || L < 1 || L > NET_MAXL || cin < 4 || cin > 64 || (cin & 3) || cout < 1 ||
        cout > 64) {
        err = "net: grid >= 1, 1 <= levels <= 4, in channels a multiple of 4 in [4, 64], out channels in [1, 64]";
        return SGLD_ERR_ARG;
    }
    n = Net();
    n.L = L;
    n.cin = cin;
    n.cout = cout;
    n.s = s;
    for (int l = 0; l < L; ++l) {
        n.width[l] = widths ? widths[l] : (l == 0 ? 16 : l == 1 ? 32 : l == 2 ? 48 : 64);
        if (n.width[l] < 4 || n.width[l] > 64 || (n.width[l] & 3)) {
            err = "net: widths must be multiples of 4 in [4, 64]";
            return SGLD_ERR_ARG;
        }
        if (l == 0) {
            n.dims[0][0] = ny;
            n.dims[0][1] = nx;
            n.dims[0][2] = nz;
        } else {
            for (int a = 0; a < 3; ++a) n.dims[l][a] = (n.dims[l - 1][a] + 1) / 2;
        }
        n.V[l] = (int64_t)n.dims[l][0] * n.dims[l][1] * n.dims[l][2];
    }
    // convolutions in parameter order
    auto add = [&](int ci, int co, int taps, int level) {
        NetConv c{ci, co, taps, level, n.nparam, n.nparam + (int64_t)taps * ci * co};
        n.nparam = c.b + co;
        n.conv.push_back(c);
    };
    for (int l = 0; l < L; ++l) {
        add(l == 0 ? cin : n.width[l - 1], n.width[l], 27, l);
        add(n.width[l], n.width[l], 27, l);
    }
    for (int l = L - 2; l >= 0; --l) {
        add(n.width[l + 1], n.width[l], 27, l + 1);
        add(n.width[l], n.width[l], 27, l);
    }
    add(n.width[0], cout, 1, 0);
    int64_t wmax = 0, pmax = 0, imax = 0;
    for (const NetConv &c : n.conv) {
        const int64_t nw = (int64_t)c.taps * c.cin * c.cout;
        wmax = std::max(wmax, nw);
        imax = std::max(imax, (int64_t)c.taps * ((c.cin + 15) & ~15) * ((c.cout + 15) & ~15));
        pmax = std::max(pmax, (int64_t)net_wgrad_splits(n.V[c.level]) * (nw + c.cout));
    }
    cudaError_t e = cudaSuccess;
#define NA(p, cnt) \
    if (e == cudaSuccess) e = nalloc(n, p, cnt)
    NA(&n.w, n.nparam);
    NA(&n.m, n.nparam);
    NA(&n.v, n.nparam);
    NA(&n.g, n.nparam);
    NA(&n.wb, n.nparam);
    NA(&n.wt, wmax);
    NA(&n.wimg, imax);
    NA(&n.tc_err, 1);
    if (e == cudaSuccess) e = cudaMemsetAsync(n.tc_err, 0, sizeof(int), s);
    NA(&n.wpart, pmax);
    NA(&n.x_own, n.V[0] * cin);
    n.X.level = 0;
    n.X.C = cin;
    for (int l = 0; l < L; ++l) {
        const int64_t nv = n.V[l] * n.width[l];
        for (NetAct *a : {&n.Ea[l], &n.E[l], &n.S[l], &n.D[l]}) {
            a->level = l;
            a->C = n.width[l];
            NA(&a->a, nv);
            NA(&a->g, nv);
        }
        if (l > 0) {   // P_l = pool(E_{l-1}) and Du_{l-1} live on level l with w_{l-1} channels
            const int64_t np = n.V[l] * n.width[l - 1];
            for (NetAct *a : {&n.P[l], &n.Du[l - 1]}) {
                a->level = l;
                a->C = n.width[l - 1];
                NA(&a->a, np);
                NA(&a->g, np);
            }
        }
    }
    NA(&n.Y, n.V[0] * cout);
    NA(&n.gY, n.V[0] * cout);
    NA(&n.T, n.V[0] * cout);
    NA(&n.M, n.V[0]);
    NA(&n.mse_part, 2 * net_mse_blocks(n.V[0]));
    NA(&n.d_loss, 1);
#undef NA
    if (e != cudaSuccess) {
        err = std::string("net: ") + cudaGetErrorString(e);
        net_free(n);
        return SGLD_ERR_CUDA;
    }
    n.X.a = n.x_own;
    net_init_attributes();
    // He-uniform weights (bound sqrt(6 / fan_in)), zero biases; the head starts
    // at a tenth of that so that the first guesses are small
    std::vector<float> h((size_t)n.nparam, 0.f);
    SplitMix rng{seed};
    for (size_t k = 0; k < n.conv.size(); ++k) {
        const NetConv &c = n.conv[k];
        const double bound = sqrt(6.0 / ((double)c.taps * c.cin)) * (k + 1 == n.conv.size() ? 0.1 : 1.0);
        for (int64_t i = c.w; i < c.b; ++i) h[(size_t)i] = (float)((2.0 * rng.uniform() - 1.0) * bound);
    }
    e = cudaMemcpyAsync(n.w, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(n.m, 0, sizeof(float) * n.nparam, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(n.v, 0, sizeof(float) * n.nparam, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(n.x_own, 0, sizeof(bf16) * n.V[0] * cin, s);
    net_to_bf16(n.w, n.wb, n.nparam, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        err = std::string("net: ") + cudaGetErrorString(e);
        net_free(n);
        return SGLD_ERR_CUDA;
    }
    return SGLD_OK;
}

void net_free(Net &n) {
    for (void *p : n.allocs) cudaFree(p);
    n.allocs.clear();
}

void net_forward(Net &n) {
    const int L = n.L;
    for (int l = 0; l < L; ++l) {
        conv_fwd(n, conv_a(l), l == 0 ? n.X.a : n.P[l].a, n.Ea[l].a, true);
        conv_fwd(n, conv_b(l), n.Ea[l].a, n.E[l].a, true);
        if (l + 1 < L) net_pool(n.E[l].a, n.width[l], n.dims[l], n.dims[l + 1], n.P[l + 1].a, n.s);
    }
    const bf16 *prev = n.E[L - 1].a;
    for (int l = L - 2; l >= 0; --l) {
        conv_fwd(n, conv_u(n, l), prev, n.Du[l].a, true);
        net_up_add(n.Du[l].a, n.E[l].a, n.width[l], n.dims[l], n.dims[l + 1], n.S[l].a, n.s);
        conv_fwd(n, conv_m(n, l), n.S[l].a, n.D[l].a, true);
        prev = n.D[l].a;
    }
    conv_fwd(n, conv_head(n), prev, n.Y, false);
}

void net_loss(Net &n, const float *T, const float *M) {
    net_mse(n.Y, T, M, n.cout, n.V[0], n.gY, n.mse_part, n.d_loss, n.s);
}

void net_backward(Net &n) {
    const int L = n.L;
    NetAct &last = L > 1 ? n.D[0] : n.E[0];
    conv_wgrad(n, conv_head(n), last.a, n.gY);
    conv_bwd(n, conv_head(n), n.gY, last.a, last.g, false);
    for (int l = 0; l <= L - 2; ++l) {
        conv_wgrad(n, conv_m(n, l), n.S[l].a, n.D[l].g);
        conv_bwd(n, conv_m(n, l), n.D[l].g, nullptr, n.S[l].g, false);
        net_up_add_bwd(n.S[l].g, n.width[l], n.dims[l], n.dims[l + 1], n.Du[l].a, n.Du[l].g, n.E[l].a, n.E[l].g,
                       false, n.s);
        NetAct &prev = (l + 1 <= L - 2) ? n.D[l + 1] : n.E[L - 1];
        conv_wgrad(n, conv_u(n, l), prev.a, n.Du[l].g);
        conv_bwd(n, conv_u(n, l), n.Du[l].g, prev.a, prev.g, false);
    }
    for (int l = L - 1; l >= 0; --l) {
        conv_wgrad(n, conv_b(l), n.Ea[l].a, n.E[l].g);
        conv_bwd(n, conv_b(l), n.E[l].g, n.Ea[l].a, n.Ea[l].g, false);
        conv_wgrad(n, conv_a(l), l == 0 ? n.X.a : n.P[l].a, n.Ea[l].g);
        if (l > 0) {
            conv_bwd(n, conv_a(l), n.Ea[l].g, nullptr, n.P[l].g, false);
            net_pool_bwd(n.P[l].g, n.width[l - 1], n.dims[l - 1], n.dims[l], n.E[l - 1].a, n.E[l - 1].g, true, n.s);
        }
    }
}

void net_adam_step(Net &n, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    ++n.step;
    const float c1 = (float)(1.0 / (1.0 - pow((double)b1, n.step)));
    const float c2 = (float)(1.0 / (1.0 - pow((double)b2, n.step)));
    net_adam(n.w, n.m, n.v, n.g, n.wb, n.nparam, lr, b1, b2, eps, c1, c2, n.s);
}

bool net_take_error(Net &n) {
    int h = 0;
    if (cudaMemcpyAsync(&h, n.tc_err, sizeof h, cudaMemcpyDeviceToHost, n.s) != cudaSuccess) return true;
    if (cudaStreamSynchronize(n.s) != cudaSuccess) return true;
    if (h && cudaMemsetAsync(n.tc_err, 0, sizeof(int), n.s) != cudaSuccess) return true;
    return h != 0;
}

}  // namespace sgld

// ---- C ABI ------------------------------------------------------------------
using namespace sgld;

struct sgld_net {
    Net n;
    std::string err;
    bool own_stream = false;
    int device = 0;   // the device current at sgld_net_create; its stream and buffers live there
};

namespace {

int nfail(sgld_net *h, int code, const std::string &m) {
    h->err = m;
    return code;
}

#define NCK(x)                                                                                       \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return nfail(h, SGLD_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// every entry point runs on the network's own device
int net_bind(sgld_net *h) {
    int dev = -1;
    NCK(cudaGetDevice(&dev));
    if (dev != h->device) NCK(cudaSetDevice(h->device));
    return SGLD_OK;
}

// host [V][cin] FP32 -> the network's BF16 input
int upload_input(sgld_net *h, const float *x) {
    Net &n = h->n;
    const int64_t cnt = n.V[0] * n.cin;
    float *tmp = nullptr;
    NCK(cudaMallocAsync((void **)&tmp, sizeof(float) * cnt, n.s));
    NCK(cudaMemcpyAsync(tmp, x, sizeof(float) * cnt, cudaMemcpyHostToDevice, n.s));
    net_to_bf16(tmp, n.x_own, cnt, n.s);
    NCK(cudaFreeAsync(tmp, n.s));
    n.X.a = n.x_own;
    return SGLD_OK;
}

int upload_target(sgld_net *h, const float *t, const float *m) {
    Net &n = h->n;
    NCK(cudaMemcpyAsync(n.T, t, sizeof(float) * n.V[0] * n.cout, cudaMemcpyHostToDevice, n.s));
    if (m) {
        NCK(cudaMemcpyAsync(n.M, m, sizeof(float) * n.V[0], cudaMemcpyHostToDevice, n.s));
    } else {
        std::vector<float> one((size_t)n.V[0], 1.f);
        NCK(cudaMemcpyAsync(n.M, one.data(), sizeof(float) * one.size(), cudaMemcpyHostToDevice, n.s));
        NCK(cudaStreamSynchronize(n.s));
    }
    return SGLD_OK;
}

}  // namespace

extern "C" {

int sgld_net_create(int ny, int nx, int nz, int in_channels, int out_channels, int levels, const int *widths,
                    unsigned long long seed, sgld_net **out) {
    if (!out) return SGLD_ERR_ARG;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SGLD_ERR_CUDA;
    sgld_net *h = new sgld_net();
    h->device = dev;
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return SGLD_ERR_CUDA;
    }
    h->own_stream = true;
    std::string err;
    const int rc = net_init(h->n, ny, nx, nz, in_channels, out_channels, levels, widths, seed, s, err);
    if (rc) {
        cudaStreamDestroy(s);
        delete h;
        return rc;
    }
    *out = h;
    return SGLD_OK;
}

void sgld_net_destroy(sgld_net *h) {
    if (!h) return;
    net_bind(h);
    if (h->n.s) cudaStreamSynchronize(h->n.s);
    net_free(h->n);
    if (h->own_stream && h->n.s) cudaStreamDestroy(h->n.s);
    delete h;
}

const char *sgld_net_last_error(const sgld_net *h) { return h ? h->err.c_str() : "null network"; }

int64_t sgld_net_num_params(const sgld_net *h) { return h ? h->n.nparam : -1; }

int sgld_net_get_params(sgld_net *h, float *w) {
    if (!h || !w) return SGLD_ERR_ARG;
    if (int rc = net_bind(h)) return rc;
    NCK(cudaMemcpyAsync(w, h->n.w, sizeof(float) * h->n.nparam, cudaMemcpyDeviceToHost, h->n.s));
    NCK(cudaStreamSynchronize(h->n.s));
    return SGLD_OK;
}

int sgld_net_set_params(sgld_net *h, const float *w) {
    if (!h || !w) return SGLD_ERR_ARG;
    if (int rc = net_bind(h)) return rc;
    Net &n = h->n;
    NCK(cudaMemcpyAsync(n.w, w, sizeof(float) * n.nparam, cudaMemcpyHostToDevice, n.s));
    net_to_bf16(n.w, n.wb, n.nparam, n.s);
    NCK(cudaMemsetAsync(n.m, 0, sizeof(float) * n.nparam, n.s));
    NCK(cudaMemsetAsync(n.v, 0, sizeof(float) * n.nparam, n.s));
    n.step = 0;
    NCK(cudaStreamSynchronize(n.s));
    return SGLD_OK;
}

int sgld_net_forward(sgld_net *h, const float *x, float *y) {
    if (!h || !x || !y) return SGLD_ERR_ARG;
    if (int rc = net_bind(h)) return rc;
    Net &n = h->n;
    int rc = upload_input(h, x);
    if (rc) return rc;
    net_forward(n);
    NCK(cudaGetLastError());
    NCK(cudaMemcpyAsync(y, n.Y, sizeof(float) * n.V[0] * n.cout, cudaMemcpyDeviceToHost, n.s));
    NCK(cudaStreamSynchronize(n.s));
    if (net_take_error(n)) return nfail(h, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up");
    return SGLD_OK;
}

int sgld_net_grad(sgld_net *h, const float *x, const float *target, const float *mask, double *loss, float *grad) {
    if (!h || !x || !target) return SGLD_ERR_ARG;
    if (int brc = net_bind(h)) return brc;
    Net &n = h->n;
    int rc = upload_input(h, x);
    if (!rc) rc = upload_target(h, target, mask);
    if (rc) return rc;
    net_forward(n);
    net_loss(n, n.T, n.M);
    net_backward(n);
    NCK(cudaGetLastError());
    if (loss) NCK(cudaMemcpyAsync(loss, n.d_loss, sizeof(double), cudaMemcpyDeviceToHost, n.s));
    if (grad) NCK(cudaMemcpyAsync(grad, n.g, sizeof(float) * n.nparam, cudaMemcpyDeviceToHost, n.s));
    NCK(cudaStreamSynchronize(n.s));
    if (net_take_error(n)) return nfail(h, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up");
    return SGLD_OK;
}

int sgld_net_train_step(sgld_net *h, const float *x, const float *target, const float *mask, float lr,
                        double *loss) {
    if (!h || !x || !target || !(lr > 0.f)) return SGLD_ERR_ARG;
    if (int brc = net_bind(h)) return brc;
    Net &n = h->n;
    int rc = upload_input(h, x);
    if (!rc) rc = upload_target(h, target, mask);
    if (rc) return rc;
    net_forward(n);
    net_loss(n, n.T, n.M);
    net_backward(n);
    net_adam_step(n, lr);
    NCK(cudaGetLastError());
    if (loss) NCK(cudaMemcpyAsync(loss, n.d_loss, sizeof(double), cudaMemcpyDeviceToHost, n.s));
    NCK(cudaStreamSynchronize(n.s));
    if (net_take_error(n)) return nfail(h, SGLD_ERR_CUDA, "a tensor-core convolution's MMA wait gave up");
    return SGLD_OK;
}

}  // extern "C"
