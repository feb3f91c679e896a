// sosfilt / sosfiltfilt for f32 data (the kernels are in sos_impl.cuh; f64
// data is instantiated in sos_f64.cu and sosfiltfilt_f64.cu).
#include "sos_impl.cuh"

namespace scir {

template int launch_sosfilt<float>(const float*, int64_t, int64_t, int64_t, const SosCoef&,
                                   const double*, double*, int, float*, int64_t, cudaStream_t,
                                   int64_t, int64_t);
template int launch_sosfiltfilt<float>(const float*, int64_t, int64_t, int64_t, const SosCoef&,
                                       int64_t, int, int, float*, int64_t, float*, cudaStream_t);

}  // namespace scir
