// Oracle driver around the reference trainer's model (test infrastructure only).
//
// Usage: ref-grad MODEL CFG [WEIGHTS]
//   Prints, as one JSON object per line:
//     {"coeffs": [...]}                               MLMTPR::Coeff() (the trained parameter vector)
//     {"cfg": c, "energy": E, "forces": [...], "stresses": [[...]], "site_energies": [...]}
//                                                     from MLMTPR::CalcEFS (dev_src/mtpr.cpp:8779)
//     {"cfg": c, "grad": [...]}                       AccumulateEFSCombinationGrad
//                                                     (src/basic_mlip.cpp:421, dev_src/mtpr.cpp:9188)
//
// Usage: ref-grad --bfgs MODEL CFG wE wF wS weighting ITERS [DIAG]
//   The reference BFGS engine over Coeff() on the trainer objective (loss / K); prints every trial
//   point and its objective value (see the mode's comment below).
//
// Usage: ref-grad --linear MODEL CFG wE wF wS [weighting]
//   MTPR_trainer::TrainLinear on the labelled CFG; prints {"coeffs": [...]} after the solve.
//
// Usage: ref-grad --rescale MODEL CFG wE wF wS [weighting]
//   Rescale (dev_src/mlp/mtpr_train.cpp:1504, the scaling search around TrainLinear) on the labelled
//   CFG as the reference trainer's training set; prints {"scaling": s, "coeffs": [...]} (its log
//   lines go to stderr).
//
// Usage: ref-grad --write MODEL OUT VALUES
//   Loads MODEL, replaces its parameter vector by the whitespace-separated VALUES (same length
//   and order as Coeff()), and saves it with MLMTPR::Save, so that the written .sus2 is in the
//   reference's own serialisation.
//
//   WEIGHTS holds, per configuration, "n" then n rows "ene_w fx fy fz" then 3 rows of the
//   3x3 stress weight; the gradient is accumulated from zero for each configuration.
#include "mtpr.h"
#include "configuration.h"
#include "non_linear_regression.h"
#include "mtpr_trainer.h"
#include "mlp/mtpr_train.h"
#include <cstdio>
#include <string>
#include <fstream>
#include <iostream>
#include <vector>

// the reference trainer's training set (a global of dev_src/mlp/mtpr_train.cpp, read by Rescale)
extern std::vector<Configuration> training_set;

static void vec(const double* v, int n) {
  std::printf("[");
  for (int i = 0; i < n; ++i) std::printf(i ? ",%.17g" : "%.17g", v[i]);
  std::printf("]");
}

int main(int argc, char** argv) {
  if (argc < 3) { std::fprintf(stderr, "usage: ref-grad MODEL CFG [WEIGHTS]\n"); return 2; }
  try {
  if (std::string(argv[1]) == "--write") {
    if (argc != 5) { std::fprintf(stderr, "usage: ref-grad --write MODEL OUT VALUES\n"); return 2; }
    MLMTPR mtpr(argv[2]);
    std::ifstream vf(argv[4]);
    std::vector<double> v;
    double x;
    while (vf >> x) v.push_back(x);
    if ((int)v.size() != mtpr.CoeffCount()) { std::fprintf(stderr, "expected %d values, got %zu\n", mtpr.CoeffCount(), v.size()); return 3; }
    for (int i = 0; i < mtpr.CoeffCount(); ++i) mtpr.Coeff()[i] = v[i];
    mtpr.DistributeCoeffs();
    mtpr.Save(argv[3]);
    return 0;
  }
  if (std::string(argv[1]) == "--loss") {
    // ref-grad --loss MODEL CFG wE wF wS [weighting [gate_x_l2]]:
    // NonLinearRegression::CalcObjectiveFunctionGrad (dev_src/non_linear_regression.cpp:1112), and
    // the error metrics it collects (energy / force / stress MAE and RMSE, :1150-1184), over
    // the labelled CFG with the energy / force / stress MSE terms only (std terms, penalties and
    // regularisers set to zero; the Effect gate-x L2 term, default 1e-4 in the reference
    // (non_linear_regression.h:128), is 0 unless given); prints the summed loss and gradient (the
    // trainer divides both by the configuration count afterwards).
    if (argc < 7) { std::fprintf(stderr, "usage: ref-grad --loss MODEL CFG wE wF wS [weighting [gate_x_l2]]\n"); return 2; }
    MLMTPR mtpr(argv[2]);
    struct Objective : NonLinearRegression {
      using NonLinearRegression::NonLinearRegression;
      double loss() const { return loss_; }
      const std::vector<double>& grad() const { return loss_grad_; }
    };
    Objective obj(&mtpr, std::stod(argv[4]), std::stod(argv[5]), std::stod(argv[6]), 0.0, 0.0);
    obj.std_scaling = 0.0;
    obj.stdd_scaling = 0.0;
    obj.radial_smooth_regularization = 0.0;
    obj.fixed_atomic_energy_weight = 0.0;
    if (argc > 7) obj.weighting = argv[7];
    obj.gate_x_l2_regularization = argc > 8 ? std::stod(argv[8]) : 0.0;
    std::ifstream in(argv[3]);
    std::vector<Configuration> train;
    Configuration c;
    while (c.Load(in)) train.push_back(c);
    obj.CalcObjectiveFunctionGrad(train);
    std::printf("{\"loss\": %.17g, \"grad\": ", obj.loss());
    vec(obj.grad().data(), (int)obj.grad().size());
    // the trainer's error metrics collected over the same pass (NonLinearRegression::EnergyMAE_meVPerAtom ...)
    const double metrics[6] = {obj.EnergyMAE_meVPerAtom(), obj.EnergyRMSE_meVPerAtom(), obj.ForceMAE_meVPerA(),
                               obj.ForceRMSE_meVPerA(), obj.StressMAE_eV(), obj.StressRMSE_eV()};
    std::printf(", \"metrics\": ");
    vec(metrics, 6);
    std::printf(", \"configs\": %zu}\n", train.size());
    return 0;
  }
  if (std::string(argv[1]) == "--bfgs") {
    // ref-grad --bfgs MODEL CFG wE wF wS weighting ITERS: the reference's BFGS engine
    // (BFGS::Iterate / Linesearch::Iterate / UpdateInvHess, src/common/bfgs.{h,cpp}) in reverse
    // communication over the raw parameter vector Coeff(), minimising the trainer objective
    // f = loss / K, g = grad / K of NonLinearRegression::CalcObjectiveFunctionGrad (the same terms
    // as --loss, gate-x term off), from the model's parameters and the identity inverse Hessian.
    // Prints, per objective evaluation, {"eval": k, "f": f, "x": [...], "accepted": a} where a says
    // whether BFGS took the evaluated point as its new line-search start; stops after ITERS
    // accepted steps beyond the starting point (or 400 evaluations).  DIAG (optional) is a file of
    // Coeff()-many values given to BFGS::SetInvHessDiagonal after Set_x, as the trainer does
    // (dev_src/mtpr_trainer.cpp:3063-3068).
    if (argc < 9) { std::fprintf(stderr, "usage: ref-grad --bfgs MODEL CFG wE wF wS weighting ITERS [DIAG]\n"); return 2; }
    MLMTPR mtpr(argv[2]);
    struct Objective : NonLinearRegression {
      using NonLinearRegression::NonLinearRegression;
      double loss() const { return loss_; }
      const std::vector<double>& grad() const { return loss_grad_; }
    };
    struct TracedBFGS : BFGS {
      const Array1D& start_x() const { return x_start; }
    };
    Objective obj(&mtpr, std::stod(argv[4]), std::stod(argv[5]), std::stod(argv[6]), 0.0, 0.0);
    obj.std_scaling = 0.0;
    obj.stdd_scaling = 0.0;
    obj.radial_smooth_regularization = 0.0;
    obj.fixed_atomic_energy_weight = 0.0;
    obj.weighting = argv[7];
    obj.gate_x_l2_regularization = 0.0;
    const int iters = std::stoi(argv[8]);
    std::ifstream in(argv[3]);
    std::vector<Configuration> train;
    Configuration c;
    while (c.Load(in)) train.push_back(c);
    const double K = static_cast<double>(train.size());
    const int n = mtpr.CoeffCount();
    TracedBFGS bfgs;
    bfgs.Set_x(mtpr.Coeff(), n);
    if (argc > 9) {
      std::ifstream df(argv[9]);
      Array1D diag(n);
      for (int i = 0; i < n; ++i)
        if (!(df >> diag[i])) { std::fprintf(stderr, "diagonal: expected %d values\n", n); return 3; }
      bfgs.SetInvHessDiagonal(diag);
    }
    Array1D g(n);
    std::vector<double> xe(n);
    int accepted = -1;
    for (int k = 0; k < 400 && accepted < iters; ++k) {
      // the trainer writes the optimiser's point straight into Coeff(), which CalcEFS reads (no
      // DistributeCoeffs: that rebuilds the readout block from the model's own copy)
      for (int i = 0; i < n; ++i) xe[i] = mtpr.Coeff()[i] = bfgs.x(i);
      obj.CalcObjectiveFunctionGrad(train);
      const double f = obj.loss() / K;
      for (int i = 0; i < n; ++i) g[i] = obj.grad()[i] / K;
      bfgs.Iterate(f, g);
      bool took = true;
      for (int i = 0; i < n && took; ++i) took = bfgs.start_x()[i] == xe[i];
      if (took) ++accepted;
      std::printf("{\"eval\": %d, \"f\": %.17g, \"accepted\": %s, \"x\": ", k, f, took ? "true" : "false");
      vec(xe.data(), n);
      std::printf("}\n");
    }
    return 0;
  }
  if (std::string(argv[1]) == "--rescale") {
    if (argc < 7) { std::fprintf(stderr, "usage: ref-grad --rescale MODEL CFG wE wF wS [weighting]\n"); return 2; }
    MLMTPR mtpr(argv[2]);
    MTPR_trainer trainer(&mtpr, std::stod(argv[4]), std::stod(argv[5]), std::stod(argv[6]));
    if (argc > 7) trainer.weighting = argv[7];
    std::ifstream in(argv[3]);
    Configuration c;
    training_set.clear();
    while (c.Load(in)) training_set.push_back(c);
    std::streambuf* keep = std::cout.rdbuf(std::cerr.rdbuf());  // the search's log lines
    Rescale(trainer, mtpr, nullptr);
    std::cout.rdbuf(keep);
    std::printf("{\"scaling\": %.17g, \"coeffs\": ", mtpr.scaling);
    vec(mtpr.Coeff(), mtpr.CoeffCount());
    std::printf(", \"configs\": %zu}\n", training_set.size());
    return 0;
  }
  if (std::string(argv[1]) == "--linear") {
    // ref-grad --linear MODEL CFG wE wF wS [weighting]: MTPR_trainer::TrainLinear
    // (dev_src/mtpr_trainer.cpp:1455) on the labelled CFG -- the linear warm-up solve of the species
    // constants and the scalar readout -- and prints the resulting parameter vector.
    if (argc < 7) { std::fprintf(stderr, "usage: ref-grad --linear MODEL CFG wE wF wS [weighting]\n"); return 2; }
    MLMTPR mtpr(argv[2]);
    MTPR_trainer trainer(&mtpr, std::stod(argv[4]), std::stod(argv[5]), std::stod(argv[6]));
    if (argc > 7) trainer.weighting = argv[7];
    std::ifstream in(argv[3]);
    std::vector<Configuration> train;
    Configuration c;
    while (c.Load(in)) train.push_back(c);
    trainer.TrainLinear(0, train, nullptr, "golden");
    std::printf("{\"coeffs\": ");
    vec(mtpr.Coeff(), mtpr.CoeffCount());
    std::printf(", \"configs\": %zu}\n", train.size());
    return 0;
  }
  MLMTPR mtpr(argv[1]);
  std::printf("{\"coeffs\": ");
  vec(mtpr.Coeff(), mtpr.CoeffCount());
  std::printf("}\n");
  std::ifstream in(argv[2]);
  std::ifstream wf;
  if (argc > 3) wf.open(argv[3]);
  Configuration cfg;
  int c = 0;
  while (cfg.Load(in)) {
    Configuration eval = cfg;
    mtpr.CalcEFS(eval);
    const int n = eval.size();
    std::printf("{\"cfg\": %d, \"energy\": %.17g, \"forces\": [", c, eval.energy);
    for (int i = 0; i < n; ++i) {
      if (i) std::printf(",");
      double f[3] = {eval.force(i)[0], eval.force(i)[1], eval.force(i)[2]};
      vec(f, 3);
    }
    std::printf("], \"stresses\": [");
    for (int a = 0; a < 3; ++a) {
      if (a) std::printf(",");
      double s[3] = {eval.stresses[a][0], eval.stresses[a][1], eval.stresses[a][2]};
      vec(s, 3);
    }
    std::printf("], \"site_energies\": ");
    vec(eval.cal_se.data(), (int)eval.cal_se.size());
    std::printf("}\n");
    if (wf.is_open()) {
      int m = 0;
      wf >> m;
      if (m != n) { std::fprintf(stderr, "weights size mismatch\n"); return 3; }
      std::vector<double> ew(n);
      std::vector<Vector3> fw(n);
      Matrix3 sw;
      for (int i = 0; i < n; ++i) wf >> ew[i] >> fw[i][0] >> fw[i][1] >> fw[i][2];
      for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) wf >> sw[a][b];
      std::vector<double> grad(mtpr.CoeffCount(), 0.0);
      Configuration g = cfg;
      mtpr.AccumulateEFSCombinationGrad(g, ew, fw, sw, grad);
      std::printf("{\"cfg\": %d, \"grad\": ", c);
      vec(grad.data(), (int)grad.size());
      std::printf("}\n");
    }
    ++c;
  }
  } catch (const MlipException& e) { std::fprintf(stderr, "reference error: %s\n", e.What()); return 1; }
  return 0;
}
