// gaugefix.cu -- placeholder until the Fourier-accelerated gauge fixer lands.
#include "../../include/glasma_gb300.h"
#include "gaugefix.h"

namespace glasma {

struct GaugeFixState {};

int gaugefix_run(GaugeFixState**, const GaugeFixArgs&, double, int, double, unsigned, double*, int* iterations,
                 std::string* err) {
  if (iterations) *iterations = 0;
  *err = "Coulomb gauge fixing not built yet";
  return GLASMA_ERR_UNSUPPORTED;
}

void gaugefix_destroy(GaugeFixState* state) { delete state; }

}  // namespace glasma
