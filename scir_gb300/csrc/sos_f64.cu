// sosfilt for f64 data (the kernels are in sos_impl.cuh; sosfiltfilt on f64
// data is instantiated in sosfiltfilt_f64.cu, both on f32 data in sos.cu).
#include "sos_impl.cuh"

namespace scir {

template int launch_sosfilt<double>(const double*, int64_t, int64_t, int64_t, const SosCoef&,
                                    const double*, double*, int, double*, int64_t, cudaStream_t,
                                    int64_t, int64_t);

}  // namespace scir
