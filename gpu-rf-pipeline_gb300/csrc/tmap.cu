// Tensor-map encoding (tmap.hpp).
#include "tmap.hpp"

#include <mutex>

namespace rfx {

namespace {

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder()
{
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult status{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &status) == cudaSuccess &&
            status == cudaDriverEntryPointSuccess) {
            fn = reinterpret_cast<EncodeTiled>(p);
        }
    });
    return fn;
}

}  // namespace

cudaError_t encode_rows_f32(CUtensorMap* map, const void* base, long long rows, int row_floats,
                            unsigned box_x, unsigned box_y)
{
    return encode_rows(map, base, 4, rows, row_floats, box_x, box_y);
}

cudaError_t encode_rows(CUtensorMap* map, const void* base, int elem_bytes, long long rows,
                        int row_elems, unsigned box_x, unsigned box_y)
{
    EncodeTiled fn = encoder();
    if (fn == nullptr) {
        return cudaErrorNotSupported;
    }
    if (rows < 1 || row_elems < 1 || box_x < 1 || box_y < 1 || box_x > 256 || box_y > 256 ||
        (elem_bytes != 4 && elem_bytes != 2 && elem_bytes != 1)) {
        return cudaErrorInvalidValue;
    }
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(row_elems),
                                static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(row_elems) *
                                   static_cast<cuuint64_t>(elem_bytes)};
    const cuuint32_t box[2] = {box_x, box_y};
    const cuuint32_t elem[2] = {1, 1};
    const CUtensorMapDataType type = elem_bytes == 4   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                     : elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                                       : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    const CUresult r = fn(map, type, 2, const_cast<void*>(base), dims,
                          strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace rfx
