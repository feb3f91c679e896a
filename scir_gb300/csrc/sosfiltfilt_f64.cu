// sosfiltfilt for f64 data (the kernels are in sos_impl.cuh; sosfilt on f64
// data is instantiated in sos_f64.cu, both on f32 data in sos.cu).
#include "sos_impl.cuh"

namespace scir {

template int launch_sosfiltfilt<double>(const double*, int64_t, int64_t, int64_t, const SosCoef&,
                                        int64_t, int, int, double*, int64_t, double*, cudaStream_t);

}  // namespace scir
