// bsa_mixed.cu -- split-precision (BF16x3) tensor-core contraction of the Classic grid.
#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

int Engine::contract_mixed(const PointSrc &ps, long long npts, double *m3mf, double *m3mr) {
    (void)ps; (void)npts; (void)m3mf; (void)m3mr;
    return fail(BSA_ERR_UNSUPPORTED, "BF16x3 contraction not available in this build");
}

int Engine::run_mesher(double *m3mf, double *m3mr) {
    (void)m3mf; (void)m3mr;
    return fail(BSA_ERR_UNSUPPORTED, "Mesher zone generation not available in this build");
}

}  // namespace bsa
