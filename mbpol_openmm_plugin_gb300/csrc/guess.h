// Learned initial guess for the induced dipoles.
//  (1) Cold starts: per-water descriptors, a 64-64-64-9 SiLU network with
//      BF16 weights on the tensor cores (mma.sync, FP32 accumulation), its
//      training (forward, backward, Adam) on the GPU, and the guess
//      mu0 = mu_prev + (m_now - m_prev) (m the network's lab-frame
//      prediction), or m_now when there is no previous solve.
//  (2) Trajectories: a linear predictor over the last solves whose
//      coefficients are refitted by least squares before every solve
//      (predictor.cu), plus a second network of the same shape (the
//      correction network) that maps each water's neighbourhood and the
//      unpredicted change of the permanent field around it to the
//      predictor's remaining error.
#pragma once
#include <cuda_runtime.h>

#include <vector>

namespace mbpol {

namespace guess {
constexpr int kFeat = 48;   // neighbourhood descriptors
constexpr int kField = 9;   // permanent field at O, H1, H2 in the water's frame
constexpr int kIn = 64;     // network input: descriptors, field, zero padding
constexpr int kHidden = 64;
constexpr int kOut = 9;
// flat parameter vector: W1 [64][64], b1 [64], W2 [64][64], b2 [64], W3 [9][64], b3 [9]
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kHidden * kIn;
constexpr int kW2 = kB1 + kHidden;
constexpr int kB2 = kW2 + kHidden * kHidden;
constexpr int kW3 = kB2 + kHidden;
constexpr int kB3 = kW3 + kOut * kHidden;
constexpr int kParams = kB3 + kOut;  // 8905
// the parameter block handed across the ABI: kParams weights, then the
// input standardisation (mean[64], 1/std[64])
constexpr int kBlockFloats = kParams + 2 * kIn;
constexpr float kOutScale = 1e-3f;  // e nm per network output unit (cold-start network)
constexpr float kResScale = 1e-7f;  // e nm per output unit of the correction network
// correction network inputs: 48 descriptors, the water's own unpredicted
// field change dF = alpha E0 - P(alpha E0) at O, H1, H2 (9, in its frame), and
// the sums over neighbouring waters B with O-O distance r < 0.6 nm of
// fc(r) dF_O(B) and fc(r) (dF_H1(B) + dF_H2(B)) (6, in its frame), one zero
constexpr int kNbField = 6;
// learned linear predictor over the history of solves (predictor.cu)
constexpr int kPredOrder = 7;    // backward differences of the dipoles in the model
constexpr int kPredRegressors = kPredOrder;  // fitted coefficients
constexpr int kPredWindow = 4;   // past steps it is fitted on
constexpr int kPredHistory = kPredOrder + 1 + kPredWindow;  // solves it needs
constexpr int kPredStats = kPredRegressors * (kPredRegressors + 1) / 2 + kPredRegressors;
// weight of the unpredicted permanent-field change: the mean response of
// the induced dipoles to it, 1 / (1 - alpha T), for liquid water; the
// 4096-water box at 0.2 fs gave 18.0, 16.8, 15.9, 15.7, 15.9 and 16.6
// solver iterations per step for 1.0, 1.6, 2.0, 2.5, 2.8 and 3.2
constexpr double kFieldGain = 2.4;
}  // namespace guess

// Converged dipoles [3n] of past solves, r[0] the newest, and the
// polarisability times the permanent field (alpha E0) of the same steps.
struct PredictorRing {
    const double* r[guess::kPredHistory];
    const double* f[guess::kPredHistory];
};
// Fits the predictor's coefficients (d_coef[kPredRegressors], device) on the
// dipole history; d_partials holds predictor_partial_blocks() x kPredStats
// doubles.
int predictor_partial_blocks();
cudaError_t predictor_fit(cudaStream_t st, int n3, const PredictorRing& ring, double* d_partials, double* d_coef);
// Starting dipoles (FP64 state and its FP32 copy) from the history, the
// coefficients and alpha E0 of the new geometry (f_now); dF (may be null)
// receives the unpredicted field change f_now - P(f).
cudaError_t predictor_apply(cudaStream_t st, int n3, const PredictorRing& ring, const double* f_now,
                            const double* d_coef, double* mu_d, float* mu_f, float* dF = nullptr);
// mu_d += m, mu_f = float(mu_d) (the correction network's output added to
// the predictor's dipoles)
cudaError_t add_correction(cudaStream_t st, int n3, const float* m, double* mu_d, float* mu_f);
// alpha E0 per dipole component, in FP64 (pol per site, E0 [sites][3]).
cudaError_t scaled_field(cudaStream_t st, int n3, const float* E0, const float* pol, double* out);

struct GuessBuffers;

// Owned by the electrostatics engine.  All arrays are device memory unless
// named h_*.
class GuessNet {
public:
    // mode 0: the cold-start network (field slots: E0; outputs: the dipoles,
    // kOutScale); mode 1: the correction network (field slots: dF and its
    // neighbour sums; outputs: the predictor's error, kResScale)
    explicit GuessNet(int mode = 0);
    ~GuessNet();
    GuessNet(const GuessNet&) = delete;
    GuessNet& operator=(const GuessNet&) = delete;

    bool ready() const { return ready_; }
    long num_samples() const { return nsamples_; }

    // network inputs D [nmol][64] (48 descriptors from the electrostatics
    // neighbour list, then mode 0: the permanent field E0 [sites][3] at O,
    // H1, H2 in the water's frame; mode 1: dF [sites][3] of the water and of
    // its neighbours as above; zeros) and frames F [nmol][9]
    cudaError_t descriptors(cudaStream_t st, int nmol, int K, const float* off, const int* nb, const float* nbd,
                            const int* nnb, int cap, const double* box, int periodic, const float* field);
    const float* d_desc() const;
    const float* d_frames() const;
    // append the current descriptors with the converged dipoles (FP64,
    // [nsites][3]; mode 1: minus the predictor's dipoles mu_base) as
    // training targets
    cudaError_t collect(cudaStream_t st, int nmol, int K, const double* mu_d, const double* mu_base = nullptr);
    // network prediction m [nsites][3] (lab frame, e nm) for the current
    // descriptors
    cudaError_t predict(cudaStream_t st, int nmol, int K, float* m_out);
    // training on the collected samples; returns the mean loss of the last
    // 10% of the steps
    cudaError_t train(cudaStream_t st, int steps, int batch, double lr, unsigned long long seed, double* loss);
    // loss, gradient and outputs for host data (n rows), no update
    cudaError_t loss_grad(cudaStream_t st, const float* h_X, const float* h_T, int n, double* loss, float* h_grad,
                          float* h_Y);
    cudaError_t get_params(float* h_block) const;
    cudaError_t set_params(const float* h_block);

    int mode() const { return mode_; }

private:
    GuessBuffers* b_;
    int mode_ = 0;
    bool ready_ = false;
    long nsamples_ = 0;
};

}  // namespace mbpol
