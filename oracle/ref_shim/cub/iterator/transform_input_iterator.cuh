/*
 * Build shim for compiling the reference's src/model.cu with CUDA 13 (TEST
 * INFRASTRUCTURE; used only by oracle/ref_build.py).
 *
 * CCCL 3 (CUDA 13) removed cub/iterator/transform_input_iterator.cuh and
 * cub::TransformInputIterator, which src/model.cu:12 includes and
 * src/model.cu:92 uses as TransformInputIterator<double, AbsVal, double*>.
 * This header supplies the same name as an alias of thrust's transform
 * iterator (value type, functor and base iterator in thrust's order).
 */
#pragma once
#include <cstddef>
#include <thrust/iterator/transform_iterator.h>

namespace cub {
template <typename ValueType, typename ConversionOp, typename InputIteratorT,
          typename OffsetT = std::ptrdiff_t>
using TransformInputIterator = thrust::transform_iterator<ConversionOp, InputIteratorT, ValueType>;
}  // namespace cub
