// bc6h_texture_unit.cu — test helper: decodes BC6H blocks with the GPU's own
// texture unit (a CUDA array of cudaChannelFormatKind{Signed,Unsigned}
// BlockCompressed6H read through a texture object, point sampling, element
// type), as an independent check of the library's host decoder.  Compiled by
// tests/test_gpu_textures.py; not part of the library.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

__global__ void k_read(cudaTextureObject_t tex, int W, int H, uint16_t* out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W || y >= H) return;
    const float4 v = tex2D<float4>(tex, x + 0.5f, y + 0.5f);
    uint16_t* o = out + 4 * ((size_t)y * W + x);
    // the decoded values are half floats: the conversion back is exact
    o[0] = __half_as_ushort(__float2half_rn(v.x));
    o[1] = __half_as_ushort(__float2half_rn(v.y));
    o[2] = __half_as_ushort(__float2half_rn(v.z));
    o[3] = __half_as_ushort(__float2half_rn(v.w));
}

// blocks: bw x bh BC6H blocks (16 bytes each, row-major); out: (4 bw) x (4 bh)
// RGBA half bit patterns.  Returns a cudaError_t value (0 = success).
extern "C" int bc6h_texture_unit_decode(const uint8_t* blocks, int bw, int bh, int is_signed, uint16_t* out) {
    const int W = 4 * bw, H = 4 * bh;
    cudaChannelFormatDesc desc = is_signed ? cudaCreateChannelDesc<cudaChannelFormatKindSignedBlockCompressed6H>()
                                           : cudaCreateChannelDesc<cudaChannelFormatKindUnsignedBlockCompressed6H>();
    cudaArray_t arr = nullptr;
    uint16_t* d_out = nullptr;
    cudaTextureObject_t tex = 0;
    cudaError_t e = cudaMallocArray(&arr, &desc, W, H);
    if (e == cudaSuccess) e = cudaMemcpy2DToArray(arr, 0, 0, blocks, (size_t)bw * 16, (size_t)bw * 16, bh,
                                                  cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        cudaResourceDesc rd = {};
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td = {};
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
    if (e == cudaSuccess) e = cudaMalloc(&d_out, (size_t)W * H * 8);
    if (e == cudaSuccess) {
        k_read<<<dim3((W + 127) / 128, H), 128>>>(tex, W, H, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, (size_t)W * H * 8, cudaMemcpyDeviceToHost);
    if (tex) cudaDestroyTextureObject(tex);
    if (d_out) cudaFree(d_out);
    if (arr) cudaFreeArray(arr);
    return (int)e;
}
