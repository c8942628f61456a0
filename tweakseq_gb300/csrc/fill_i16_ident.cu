// fill_i16_ident.cu -- the int16x2 fill for identity counts (global), plain and
// overflow-checked (one translation unit per output mode so they compile in
// parallel).
#include "fill_i16.cuh"

namespace tsq {
namespace fill {

template cudaError_t launch_i16<kOutIdent>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
template int occupancy_i16<kOutIdent>(bool, bool, size_t);

}  // namespace fill
}  // namespace tsq
