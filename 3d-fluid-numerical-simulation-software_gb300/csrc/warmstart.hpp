// Learned warm start: a coordinate MLP that maps a cell centre and the operating point of a case
// to the conserved variables (and the eddy viscosity) of a converged field, trained on fields
// this solver produced, evaluated on the device to give a new case its starting field. BF16
// operands with FP32 accumulation on the fifth-generation tensor cores (tcgen05, TMEM
// accumulators); FP32 master weights and Adam moments.
//
// Network: 64 inputs (Fourier features sin / cos(pi 2^f c) f = 0..7 of the normalised axial
// position, radius and pitch angle of the cell centre, the three normalised coordinates, the
// three normalised case parameters, zeros) -> 5 hidden layers of 256 with SiLU -> 16 outputs of
// which the first six are (rho, rho u, rho v, rho w, rho E, mu_t), normalised by the training
// set's mean and standard deviation.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include "solver.hpp"

namespace gbt {

constexpr int kWsIn = 64, kWsHidden = 256, kWsOut = 16, kWsOutUsed = 6, kWsLayers = 6;
constexpr int kWsParams = 3;                     // case parameters per case
constexpr int kWsNorm = 24;                      // coord min[3], max[3]; param mean[3], std[3]; target mean[6], std[6]

class WarmStart {
public:
    explicit WarmStart(unsigned seed);
    ~WarmStart();
    WarmStart(const WarmStart &) = delete;
    WarmStart &operator=(const WarmStart &) = delete;

    // appends every fine-level interior cell of every case of the solver (its current state) to
    // the training set; params: kWsParams values per case
    void add_solves(SolverBase &s, const float *params);
    long long samples() const { return n_set; }
    // Adam steps on random minibatches; returns the mean loss of the last (up to) 20 steps. The
    // normalisation constants are computed from the training set at the first call.
    float train(int steps, int batch, float lr);
    // the network's field on the fine level of every case, kept for a case when its initial
    // residual is below the uniform start's (used[case] = 1), else the uniform start (0)
    void apply(SolverBase &s, const float *params, int *used, double *res_warm, double *res_uniform);

    static size_t n_params();
    void get_params(float *out);
    void set_params(const float *in);
    void get_norm(float *out) const;
    void set_norm(const float *in);
    // the network on given features (M x kWsIn): outputs (M x kWsOut); with targets (M x 6,
    // normalised), the loss and the gradient of every parameter (n_params values)
    void forward(const float *feat, int M, float *y);
    float forward_backward(const float *feat, const float *target, int M, float *grad);
    // device time (CUDA events on the network's stream) per layer-by-layer forward pass, per
    // forward and backward pass and per fused inference pass over M rows of device-resident random
    // features and targets, mean of iters; max_diff: the largest difference between the fused and
    // the layer-by-layer outputs
    void benchmark(long long M, int iters, float *ms_forward, float *ms_step, float *ms_infer, double *max_diff);
    int error_flag();

private:
    struct Impl;
    Impl *d;
    long long n_set = 0;
};

}  // namespace gbt
