// bc7_texture_unit.cu — test helper: decodes BC7 blocks with the GPU's own
// texture unit (a CUDA array of cudaChannelFormatKindUnsignedBlockCompressed7
// read through a texture object), as an independent check of the library's
// host decoder.  Compiled by tests/test_gpu_textures.py; not part of the
// library.
#include <cuda_runtime.h>
#include <stdint.h>

__global__ void k_read(cudaTextureObject_t tex, int W, int H, uint8_t* out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W || y >= H) return;
    const float4 v = tex2D<float4>(tex, x + 0.5f, y + 0.5f);
    uint8_t* o = out + 4 * ((size_t)y * W + x);
    o[0] = (uint8_t)__float2int_rn(v.x * 255.0f);
    o[1] = (uint8_t)__float2int_rn(v.y * 255.0f);
    o[2] = (uint8_t)__float2int_rn(v.z * 255.0f);
    o[3] = (uint8_t)__float2int_rn(v.w * 255.0f);
}

// blocks: bw x bh BC7 blocks (16 bytes each, row-major); out: (4 bw) x (4 bh) RGBA8.
// Returns a cudaError_t value (0 = success).
extern "C" int bc7_texture_unit_decode(const uint8_t* blocks, int bw, int bh, uint8_t* out) {
    const int W = 4 * bw, H = 4 * bh;
    cudaChannelFormatDesc desc = cudaCreateChannelDesc<cudaChannelFormatKindUnsignedBlockCompressed7>();
    cudaArray_t arr = nullptr;
    uint8_t* d_out = nullptr;
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
        td.readMode = cudaReadModeNormalizedFloat;
        td.normalizedCoords = 0;
        e = cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
    if (e == cudaSuccess) e = cudaMalloc(&d_out, (size_t)W * H * 4);
    if (e == cudaSuccess) {
        k_read<<<dim3((W + 127) / 128, H), 128>>>(tex, W, H, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, (size_t)W * H * 4, cudaMemcpyDeviceToHost);
    if (tex) cudaDestroyTextureObject(tex);
    if (d_out) cudaFree(d_out);
    if (arr) cudaFreeArray(arr);
    return (int)e;
}
