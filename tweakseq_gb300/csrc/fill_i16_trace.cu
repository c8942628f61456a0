// fill_i16_trace.cu -- the int16x2 fill for traceback planes (global and local), plain and
// overflow-checked (one translation unit per output mode so they compile in
// parallel).
#include "fill_i16.cuh"

namespace tsq {
namespace fill {

template cudaError_t launch_i16<kOutTrace>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
template int occupancy_i16<kOutTrace>(bool, bool, size_t);

}  // namespace fill
}  // namespace tsq
