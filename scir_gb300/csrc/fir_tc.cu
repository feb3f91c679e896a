// Tensor-core (tcgen05) FIR and polyphase contraction with split-bf16 operands.
#include "common.cuh"
#include "kernels.cuh"

namespace scir {

bool fir_tc_supported(const FirArgs&) { return false; }
int launch_fir_tc(const FirArgs&, int, cudaStream_t) {
    return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core FIR not built");
}
bool poly_tc_supported(const PolyArgs&) { return false; }
int launch_poly_tc(const PolyArgs&, int, cudaStream_t) {
    return set_error(SCIR_ERR_UNSUPPORTED, "tensor-core polyphase not built");
}

}  // namespace scir
