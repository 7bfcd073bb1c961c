/* Host stand-in for the reference's BatchedLASolver (include/batched_la.cuh:10-30)
 * used only when the reference is compiled for the CPU (oracle/build_ref.sh):
 * cuSOLVER/cuBLAS need a GPU.  lsq_svd keeps the reference's contract
 * (src/batched_la.cu:152-178): x = V diag(s_i > tol*s_max ? 1/s_i : 0) U^T b per
 * 3x3 system; for the symmetric systems DC builds, the singular values are
 * |eigenvalues|.  Solved in FP64 by cyclic Jacobi (Golub & Van Loan 8.5).
 * TEST INFRASTRUCTURE ONLY. */
#include "batched_la.cuh"

#include <cmath>

BatchedLASolver::BatchedLASolver() {}
BatchedLASolver::~BatchedLASolver() {}

static void jacobi3(double a[3][3], double w[3], double q[3][3]) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) q[i][j] = (i == j);
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = a[0][1] * a[0][1] + a[0][2] * a[0][2] + a[1][2] * a[1][2];
        double tot = off + a[0][0] * a[0][0] + a[1][1] * a[1][1] + a[2][2] * a[2][2];
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int r = p + 1; r < 3; r++) {
                if (a[p][r] == 0.0) continue;
                double th = (a[r][r] - a[p][p]) / (2.0 * a[p][r]);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    double x = a[k][p], y = a[k][r];
                    a[k][p] = c * x - s * y; a[k][r] = s * x + c * y;
                }
                for (int k = 0; k < 3; k++) {
                    double x = a[p][k], y = a[r][k];
                    a[p][k] = c * x - s * y; a[r][k] = s * x + c * y;
                }
                for (int k = 0; k < 3; k++) {
                    double x = q[k][p], y = q[k][r];
                    q[k][p] = c * x - s * y; q[k][r] = s * x + c * y;
                }
            }
    }
    for (int i = 0; i < 3; i++) w[i] = a[i][i];
}

std::tuple<NDArray<float>, NDArray<int>>
BatchedLASolver::lsq_svd(const NDArray<float> &A, const NDArray<float> &b, float tol) {
    size_t batch = A.shape[0];
    NDArray<float> x({batch, 3});
    NDArray<int> info({batch});
    const float *pa = A.data(), *pb = b.data();
    float *px = x.data();
    int *pi = info.data();
    for (size_t i = 0; i < batch; i++) {
        double a[3][3], w[3], q[3][3], r[3] = {0, 0, 0}, smax = 0;
        for (int u = 0; u < 3; u++)
            for (int v = 0; v < 3; v++) a[u][v] = pa[9 * i + 3 * u + v];
        jacobi3(a, w, q);
        for (int k = 0; k < 3; k++) smax = std::fmax(smax, std::fabs(w[k]));
        for (int k = 0; k < 3; k++) {
            float sk = (float)std::fabs(w[k]);
            if (!(sk > tol * (float)smax)) continue;
            double qb = q[0][k] * pb[3 * i] + q[1][k] * pb[3 * i + 1] + q[2][k] * pb[3 * i + 2];
            for (int m = 0; m < 3; m++) r[m] += qb / w[k] * q[m][k];
        }
        for (int m = 0; m < 3; m++) px[3 * i + m] = (float)r[m];
        pi[i] = 0;
    }
    return {std::move(x), std::move(info)};
}
