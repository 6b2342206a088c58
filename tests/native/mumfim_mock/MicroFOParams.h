// Stand-in for the solution-strategy records of mumfim's MicroFOParams.h:
// the two fields of the explicit strategy the shim reads. Test
// infrastructure only.
#ifndef MFG_TEST_MICRO_FO_PARAMS_H
#define MFG_TEST_MICRO_FO_PARAMS_H
namespace mumfim {
struct MicroSolutionStrategy {
  virtual ~MicroSolutionStrategy() = default;
  double cnvgTolerance = 1e-6;
};
struct MicroSolutionStrategyExplicit : MicroSolutionStrategy {
  double visc_damp_coeff = 0.5;
  double crit_time_scale_factor = 0.8;
};
}  // namespace mumfim
#endif
