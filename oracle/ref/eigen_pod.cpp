// C-ABI driver of the reference's POD arithmetic, built against the vendored Eigen 3.3.7
// of the reference tree (solvers/IncNavierStokesSolver/EquationSystems/ThirdParty/Eigen,
// header-only, included in place). TEST INFRASTRUCTURE: it computes what
// CoupledLinearNS_ROM::ROM_offline_phase / ROM_online_phase compute, so that the golden
// POD fixtures hold the reference's own numbers.
//   ref_pod_bdcsvd           Eigen::BDCSVD<MatrixXd>(S, ComputeThinU): singular values and
//                            the leading left singular vectors (CoupledLinearNS_ROM.cpp:3925-3954)
//   ref_pod_colpivqr_solve   MatrixXd::colPivHouseholderQr().solve(b) (:4053)
#include "Eigen/Dense"

extern "C" {

// S: N x ns column-major. sigma: ns values; U: N x nmodes column-major (the first nmodes
// columns of the thin U).
int ref_pod_bdcsvd(int N, int ns, const double* S, int nmodes, double* sigma, double* U) {
  if (N <= 0 || ns <= 0 || nmodes < 0 || nmodes > ns || nmodes > N) return 1;
  Eigen::Map<const Eigen::MatrixXd> Sm(S, N, ns);
  Eigen::BDCSVD<Eigen::MatrixXd> svd(Sm, Eigen::ComputeThinU);
  const Eigen::VectorXd sv = svd.singularValues();
  for (int i = 0; i < (int)sv.size(); ++i) sigma[i] = sv(i);
  const Eigen::MatrixXd Uf = svd.matrixU();
  Eigen::Map<Eigen::MatrixXd> Um(U, N, nmodes);
  Um = Uf.leftCols(nmodes);
  return 0;
}

// A: r x r column-major; x = A^-1 b by column-pivoted Householder QR.
int ref_pod_colpivqr_solve(int r, const double* A, const double* b, double* x) {
  if (r <= 0) return 1;
  Eigen::Map<const Eigen::MatrixXd> Am(A, r, r);
  Eigen::Map<const Eigen::VectorXd> bm(b, r);
  const Eigen::VectorXd xs = Am.colPivHouseholderQr().solve(bm);
  for (int i = 0; i < r; ++i) x[i] = xs(i);
  return 0;
}

}  // extern "C"
