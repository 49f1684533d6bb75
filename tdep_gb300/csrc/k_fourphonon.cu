// Four-phonon scattering kernel (scattering_fourphonon.f90). Not yet implemented on the
// device: the entry point reports cudaErrorNotSupported and tdg_scattering refuses
// --fourthorder with TDG_ERR_PARAM.
#include "tdg_internal.cuh"

namespace tdg {

cudaError_t launch_fourphonon(const FourPhArgs &, int, int, cudaStream_t) { return cudaErrorNotSupported; }

}  // namespace tdg
