// DoubleMLP u- 2x16, u+ 2x16 (tanh): residual-path kernels for this shape.
#define DIPS_LM 2
#define DIPS_WM 16
#define DIPS_LP 2
#define DIPS_WP 16
#define DIPS_NS arch_2_16_2_16
#define DIPS_GETTER arch_ops_2_16_2_16
#include "residual_arch.cuh"
