// selftest.cu -- the device prefix sum and radix sort (k_scan.cuh) on host
// arrays, for tests against host results.
#include "../../include/dio_cuda.h"
#include "../../include/dio_selftest.h"
#include <vector>

#include "k_scan.cuh"

namespace {

struct Run {
    cudaStream_t s = nullptr;
    dio::ScanSort ss;
    uint32_t* err = nullptr;
    std::vector<void*> bufs;
    cudaError_t e = cudaSuccess;
    ~Run() {
        if (s) cudaStreamSynchronize(s);
        ss.release();
        for (void* p : bufs) cudaFree(p);
        if (err) cudaFree(err);
        if (s) cudaStreamDestroy(s);
    }
    template <class T>
    T* dev(size_t n) {
        void* p = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T));
        if (p) bufs.push_back(p);
        return static_cast<T*>(p);
    }
    bool ok(cudaError_t r) {
        if (e == cudaSuccess) e = r;
        return e == cudaSuccess;
    }
    int start(uint32_t max_sort, uint32_t max_scan) {
        if (!ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking))) return DIO_ERR_CUDA;
        if (!ok(cudaMalloc(&err, 4)) || !ok(cudaMemsetAsync(err, 0, 4, s))) return DIO_ERR_CUDA;
        if (!ok(ss.init(max_sort, max_scan, err, s))) return DIO_ERR_CUDA;
        return DIO_OK;
    }
    int finish() {
        uint32_t flags = 0;
        if (!ok(cudaMemcpyAsync(&flags, err, 4, cudaMemcpyDeviceToHost, s)) || !ok(cudaStreamSynchronize(s)))
            return DIO_ERR_CUDA;
        return (flags & dio::kErrTimeout) ? DIO_ERR_TIMEOUT : DIO_OK;
    }
};

template <class K>
int sort_t(const K* keys, const uint32_t* vals, uint32_t n, uint32_t begin_bit, uint32_t end_bit, K* keys_out,
           uint32_t* vals_out) {
    if (n && (!keys || !vals || !keys_out || !vals_out)) return DIO_ERR_INVALID;
    if (end_bit > 8 * sizeof(K) || begin_bit > end_bit) return DIO_ERR_INVALID;
    if (n == 0) return DIO_OK;
    Run r;
    int rc = r.start(n, 1);
    if (rc) return rc;
    K* dk = r.dev<K>(n);
    K* dko = r.dev<K>(n);
    uint32_t* dv = r.dev<uint32_t>(n);
    uint32_t* dvo = r.dev<uint32_t>(n);
    if (!r.ok(r.e)) return DIO_ERR_CUDA;
    if (!r.ok(cudaMemcpyAsync(dk, keys, (size_t)n * sizeof(K), cudaMemcpyHostToDevice, r.s)) ||
        !r.ok(cudaMemcpyAsync(dv, vals, (size_t)n * 4, cudaMemcpyHostToDevice, r.s)) ||
        !r.ok(r.ss.sort_pairs(dk, dko, dv, dvo, n, begin_bit, end_bit, false, r.s)) ||
        !r.ok(cudaMemcpyAsync(keys_out, dko, (size_t)n * sizeof(K), cudaMemcpyDeviceToHost, r.s)) ||
        !r.ok(cudaMemcpyAsync(vals_out, dvo, (size_t)n * 4, cudaMemcpyDeviceToHost, r.s)))
        return DIO_ERR_CUDA;
    return r.finish();
}

}  // namespace

extern "C" {

int dio_selftest_scan(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t live, uint32_t repeats,
                      uint32_t* total) {
    if ((n && (!in || !out)) || repeats == 0) return DIO_ERR_INVALID;
    Run r;
    int rc = r.start(1, std::max(n, 1u));
    if (rc) return rc;
    uint32_t* di = r.dev<uint32_t>(n);
    uint32_t* dout = r.dev<uint32_t>(n);
    uint32_t* dlive = r.dev<uint32_t>(2);  // live count, total
    if (!r.ok(r.e)) return DIO_ERR_CUDA;
    const uint32_t head[2] = {live, 0u};
    if (!r.ok(cudaMemcpyAsync(dlive, head, 8, cudaMemcpyHostToDevice, r.s))) return DIO_ERR_CUDA;
    if (n && (!r.ok(cudaMemcpyAsync(di, in, (size_t)n * 4, cudaMemcpyHostToDevice, r.s)) ||
              !r.ok(cudaMemcpyAsync(dout, out, (size_t)n * 4, cudaMemcpyHostToDevice, r.s))))
        return DIO_ERR_CUDA;
    for (uint32_t k = 0; k < repeats; ++k)
        if (!r.ok(r.ss.scan(di, dout, n, k > 0, r.s, dlive, dlive + 1))) return DIO_ERR_CUDA;
    uint32_t tail[2] = {0u, 0u};
    if (n && !r.ok(cudaMemcpyAsync(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost, r.s))) return DIO_ERR_CUDA;
    if (!r.ok(cudaMemcpyAsync(tail, dlive, 8, cudaMemcpyDeviceToHost, r.s))) return DIO_ERR_CUDA;
    rc = r.finish();
    if (total) *total = tail[1];
    return rc;
}

int dio_selftest_sort_u32(const uint32_t* keys, const uint32_t* vals, uint32_t n, uint32_t begin_bit,
                          uint32_t end_bit, uint32_t* keys_out, uint32_t* vals_out) {
    return sort_t<uint32_t>(keys, vals, n, begin_bit, end_bit, keys_out, vals_out);
}

int dio_selftest_sort_u64(const uint64_t* keys, const uint32_t* vals, uint32_t n, uint32_t begin_bit,
                          uint32_t end_bit, uint64_t* keys_out, uint32_t* vals_out) {
    static_assert(sizeof(uint64_t) == sizeof(unsigned long long), "64-bit keys");
    return sort_t<unsigned long long>(reinterpret_cast<const unsigned long long*>(keys), vals, n, begin_bit, end_bit,
                                      reinterpret_cast<unsigned long long*>(keys_out), vals_out);
}

}  // extern "C"
