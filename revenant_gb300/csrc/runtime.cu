// Runtime half of the C ABI: context, buffers, errors.
//
// Stands in for core/gpu/context.{h,cpp} (device pick by index or
// REVENANT_GPU_INDEX, device limits, one submission queue) and
// core/gpu/buffer.{h,cpp} (DeviceLocal / Upload / Readback memory kinds),
// over the CUDA runtime. A context owns one non-blocking stream, the
// equivalent of the reference's single compute queue.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <string>

#include "common.cuh"
#include "revenant_gb300.h"

namespace rv {

static thread_local std::string g_last_error;

int32_t set_error(int32_t code, const std::string& message) {
    g_last_error = message;
    return code;
}

int32_t set_error_fmt(int32_t code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int32_t clear_error() {
    g_last_error.clear();
    return RV_OK;
}

int32_t cuda_status(cudaError_t err, const char* what) {
    if (err == cudaSuccess) return RV_OK;
    const int32_t code = (err == cudaErrorMemoryAllocation) ? RV_ERR_NO_MEMORY : RV_ERR_CUDA;
    return set_error_fmt(code, "%s: %s (%s)", what, cudaGetErrorString(err), cudaGetErrorName(err));
}

}  // namespace rv

// A context lives until it has been destroyed AND every buffer made from it
// is gone: buffers hold a reference, so destroying a context before its
// buffers (in any order a caller or a garbage collector picks) is safe.
struct rv_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    rv_device_info info{};
    std::mutex lock;
    int references = 1;  // the creator's
    bool destroyed = false;
};

namespace {
void release(rv_context* ctx) {
    bool last;
    {
        std::lock_guard<std::mutex> g(ctx->lock);
        last = --ctx->references == 0;
    }
    if (last) delete ctx;
}
}  // namespace

struct rv_buffer {
    rv_context* context = nullptr;
    void* address = nullptr;
    uint64_t bytes = 0;
    int32_t kind = RV_MEMORY_DEVICE_LOCAL;
};

using rv::cuda_status;
using rv::set_error_fmt;

extern "C" {

const char* rv_last_error(void) { return rv::g_last_error.c_str(); }

int32_t rv_abi_version(void) { return RV_ABI_VERSION; }

int32_t rv_context_create(int32_t device_index, rv_context** out) {
    if (out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_context_create: out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t err = cudaGetDeviceCount(&count);
    if (err != cudaSuccess || count == 0)
        return set_error_fmt(RV_ERR_NO_DEVICE, "rv_context_create: no CUDA device (%s)",
                             cudaGetErrorString(err));
    int device = device_index;
    if (device < 0) {
        // core/gpu/context.cpp:174 REVENANT_GPU_INDEX
        const char* env = getenv("REVENANT_GPU_INDEX");
        device = env ? atoi(env) : 0;
    }
    if (device < 0 || device >= count)
        return set_error_fmt(RV_ERR_NO_DEVICE, "rv_context_create: device %d of %d", device, count);
    cudaDeviceProp prop;
    if (int32_t st = cuda_status(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties"))
        return st;
    if (prop.major < 10)
        return set_error_fmt(RV_ERR_NO_DEVICE,
                             "rv_context_create: %s is sm_%d%d; this library is built for sm_103a",
                             prop.name, prop.major, prop.minor);
    if (int32_t st = cuda_status(cudaSetDevice(device), "cudaSetDevice")) return st;
    rv_context* ctx = new (std::nothrow) rv_context;
    if (ctx == nullptr) return set_error_fmt(RV_ERR_NO_MEMORY, "rv_context_create: out of host memory");
    ctx->device = device;
    if (int32_t st = cuda_status(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking),
                                 "cudaStreamCreate")) {
        delete ctx;
        return st;
    }
    snprintf(ctx->info.name, sizeof ctx->info.name, "%s", prop.name);
    ctx->info.device_index = device;
    ctx->info.sm_count = prop.multiProcessorCount;
    ctx->info.cc_major = prop.major;
    ctx->info.cc_minor = prop.minor;
    ctx->info.total_memory = prop.totalGlobalMem;
    ctx->info.max_shared_per_block = prop.sharedMemPerBlockOptin;
    ctx->info.l2_bytes = prop.l2CacheSize;
    *out = ctx;
    return rv::clear_error();
}

int32_t rv_context_destroy(rv_context* ctx) {
    if (ctx == nullptr) return RV_OK;
    {
        std::lock_guard<std::mutex> g(ctx->lock);
        if (ctx->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_context_destroy: already destroyed");
        ctx->destroyed = true;
    }
    cudaSetDevice(ctx->device);
    if (ctx->stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        ctx->stream = nullptr;
    }
    release(ctx);
    return rv::clear_error();
}

int32_t rv_context_device_info(const rv_context* ctx, rv_device_info* out) {
    if (ctx == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_context_device_info: NULL");
    *out = ctx->info;
    return rv::clear_error();
}

void* rv_context_stream(const rv_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int32_t rv_stream_create(rv_context* ctx, void** out) {
    if (ctx == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_stream_create: NULL");
    *out = nullptr;
    cudaStream_t s = nullptr;
    if (int32_t st = cuda_status(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate")) return st;
    *out = (void*)s;
    return rv::clear_error();
}

int32_t rv_stream_destroy(void* stream) {
    if (stream == nullptr) return RV_OK;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaStreamSynchronize(s);
    if (int32_t st = cuda_status(cudaStreamDestroy(s), "cudaStreamDestroy")) return st;
    return rv::clear_error();
}

int32_t rv_stream_synchronize(void* stream) {
    if (int32_t st = cuda_status(cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream)), "cudaStreamSynchronize"))
        return st;
    return rv::clear_error();
}

int32_t rv_context_synchronize(rv_context* ctx) {
    if (ctx == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_context_synchronize: NULL");
    if (int32_t st = cuda_status(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize")) return st;
    return rv::clear_error();
}

int32_t rv_buffer_create(rv_context* ctx, uint64_t bytes, int32_t kind, rv_buffer** out) {
    if (ctx == nullptr || out == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_create: NULL");
    *out = nullptr;
    if (ctx->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_create: context was destroyed");
    if (bytes == 0) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_create: zero bytes");
    void* address = nullptr;
    cudaError_t err;
    switch (kind) {
        case RV_MEMORY_DEVICE_LOCAL: err = cudaMalloc(&address, bytes); break;
        case RV_MEMORY_UPLOAD: err = cudaHostAlloc(&address, bytes, cudaHostAllocWriteCombined); break;
        case RV_MEMORY_READBACK: err = cudaHostAlloc(&address, bytes, cudaHostAllocDefault); break;
        default: return set_error_fmt(RV_ERR_INVALID, "rv_buffer_create: unknown memory kind %d", kind);
    }
    if (int32_t st = cuda_status(err, "rv_buffer_create")) return st;
    rv_buffer* b = new (std::nothrow) rv_buffer;
    if (b == nullptr) {
        if (kind == RV_MEMORY_DEVICE_LOCAL) cudaFree(address);
        else cudaFreeHost(address);
        return set_error_fmt(RV_ERR_NO_MEMORY, "rv_buffer_create: out of host memory");
    }
    {
        std::lock_guard<std::mutex> g(ctx->lock);
        ctx->references += 1;
    }
    b->context = ctx;
    b->address = address;
    b->bytes = bytes;
    b->kind = kind;
    *out = b;
    return rv::clear_error();
}

int32_t rv_buffer_destroy(rv_buffer* b) {
    if (b == nullptr) return RV_OK;
    rv_context* ctx = b->context;
    cudaSetDevice(ctx->device);
    // cudaFree / cudaFreeHost wait for outstanding work on the buffer
    if (b->kind == RV_MEMORY_DEVICE_LOCAL) cudaFree(b->address);
    else cudaFreeHost(b->address);
    delete b;
    release(ctx);
    return rv::clear_error();
}

void* rv_buffer_address(const rv_buffer* b) { return b ? b->address : nullptr; }
uint64_t rv_buffer_size(const rv_buffer* b) { return b ? b->bytes : 0; }

int32_t rv_buffer_upload(rv_buffer* b, uint64_t offset, const void* src, uint64_t bytes) {
    if (b == nullptr || src == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_upload: NULL");
    if (offset > b->bytes || bytes > b->bytes - offset)
        return set_error_fmt(RV_ERR_INVALID, "rv_buffer_upload: [%llu, +%llu) outside a %llu-byte buffer",
                             (unsigned long long)offset, (unsigned long long)bytes,
                             (unsigned long long)b->bytes);
    char* dst = static_cast<char*>(b->address) + offset;
    if (b->context->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_upload: context was destroyed");
    if (b->kind != RV_MEMORY_DEVICE_LOCAL) {
        memcpy(dst, src, bytes);
        return rv::clear_error();
    }
    if (int32_t st = cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->context->stream),
                                 "rv_buffer_upload"))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(b->context->stream), "rv_buffer_upload sync")) return st;
    return rv::clear_error();
}

int32_t rv_buffer_download(const rv_buffer* b, uint64_t offset, void* dst, uint64_t bytes) {
    if (b == nullptr || dst == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_download: NULL");
    if (offset > b->bytes || bytes > b->bytes - offset)
        return set_error_fmt(RV_ERR_INVALID, "rv_buffer_download: range outside the buffer");
    const char* src = static_cast<const char*>(b->address) + offset;
    if (b->context->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_download: context was destroyed");
    if (b->kind != RV_MEMORY_DEVICE_LOCAL) {
        memcpy(dst, src, bytes);
        return rv::clear_error();
    }
    if (int32_t st = cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, b->context->stream),
                                 "rv_buffer_download"))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(b->context->stream), "rv_buffer_download sync"))
        return st;
    return rv::clear_error();
}

int32_t rv_buffer_clear(rv_buffer* b) {
    if (b == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_clear: NULL");
    if (b->context->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_buffer_clear: context was destroyed");
    if (b->kind != RV_MEMORY_DEVICE_LOCAL) {
        memset(b->address, 0, b->bytes);
        return rv::clear_error();
    }
    if (int32_t st = cuda_status(cudaMemsetAsync(b->address, 0, b->bytes, b->context->stream), "rv_buffer_clear"))
        return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(b->context->stream), "rv_buffer_clear sync")) return st;
    return rv::clear_error();
}

int32_t rv_copy(rv_context* ctx, void* dst, const void* src, uint64_t bytes) {
    if (ctx == nullptr || dst == nullptr || src == nullptr) return set_error_fmt(RV_ERR_INVALID, "rv_copy: NULL");
    if (ctx->destroyed) return set_error_fmt(RV_ERR_INVALID, "rv_copy: context was destroyed");
    if (bytes == 0) return rv::clear_error();
    if (int32_t st = cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, ctx->stream), "rv_copy")) return st;
    if (int32_t st = cuda_status(cudaStreamSynchronize(ctx->stream), "rv_copy sync")) return st;
    return rv::clear_error();
}

}  // extern "C"
