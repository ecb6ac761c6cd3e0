// Tensor-core (tcgen05) FP32-emulating GEMMs for the mixed-precision
// factorizations: 3xTF32 and 3xBF16 split products with FP32 accumulation in
// TMEM.
#include "common.cuh"

namespace ddla {

int gemm_tc(ddla_handle h, int prec, i64 m, i64 n, i64 k, float alpha, View<const float> A, View<const float> B,
            float beta, View<float> C, int uplo) {
    (void)h; (void)prec; (void)m; (void)n; (void)k; (void)alpha; (void)A; (void)B; (void)beta; (void)C; (void)uplo;
    set_error("tensor-core split-precision GEMM not available in this build");
    return DDLA_ERR_UNSUPPORTED;
}

int gemm_ozaki(ddla_handle h, i64 m, i64 n, i64 k, double alpha, View<const double> A, View<const double> B,
               double beta, View<double> C, int prec) {
    (void)h; (void)m; (void)n; (void)k; (void)alpha; (void)A; (void)B; (void)beta; (void)C; (void)prec;
    set_error("split-precision FP64 GEMM not available in this build");
    return DDLA_ERR_UNSUPPORTED;
}

}  // namespace ddla
