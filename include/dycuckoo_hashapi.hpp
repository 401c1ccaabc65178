// dycuckoo_hashapi.hpp -- the reference's host class hashAPI
// (pauline-ly/databases_gpu GPU/dyhash/api.h:9-54, api.cpp) rebuilt on the
// C ABI of dycuckoo.h. A program written against the reference's api.h keeps
// its calls; it includes this header instead and links -ldycuckoo.
//
// Same names and argument meaning as the reference. Behaviour differences,
// all deliberate and listed here:
//   * failures throw dycuckoo::error (the reference prints via
//     checkCudaErrors and continues);
//   * hash_insert is an upsert and never drops an entry (the reference adds
//     a second copy of a repeated key and drops the entry left at the end of
//     a 15-step eviction chain, cuckoo.cu:377-431);
//   * hash_delete leaves zeros in ans like the reference and returns the
//     number of keys removed;
//   * any number of hashAPI objects may live at once (the reference keeps
//     its table in one __constant__ symbol, cuckoo.cu:16);
//   * num_size is the exact live count (the reference counts nominal batch
//     sizes, api.cpp:371, :490);
//   * the 4 GiB the reference's CNMeM pool takes at construction are mapped
//     into the library's stream-ordered pool instead (dyc_pool_reserve).
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "dycuckoo.h"

namespace dycuckoo {

using TYPE = unsigned int;  // GPU/dyhash/dy_hash.h:16

// GPU/dyhash/test_uilt.h:1-5
constexpr double kUpperBound = 0.8;
constexpr double kLowerBound = 0.5;
constexpr int BATCH_NUM = 1000;
constexpr int BATCH_SIZE = 100000;
// GPU/dyhash/api.cpp:496
constexpr double kMinDownsizeCapacity = 4 * 1024 * 1024 * 1.2;

class error : public std::runtime_error {
  public:
    error(const char *where, dyc_status s)
        : std::runtime_error(std::string(where) + ": " + dyc_status_string(s) + ": " +
                             dyc_last_error()),
          status(s) {}
    dyc_status status;
};

inline void check(dyc_status s, const char *where) {
    if (s != DYC_OK) throw error(where, s);
}

class hashAPI {
  public:
    // api.cpp:26-91. Plain hash_insert applies no load-factor check (the
    // reference compiles it out, api.cpp:185-194); the batch calls do.
    // Both constructors map 4 GiB into the library's allocation pool, as the
    // reference's constructor sizes its CNMeM pool (api.cpp:37-40), so the
    // first resizes do not map memory inside a call.
    explicit hashAPI(TYPE size) {
        dyc_config cfg;
        dyc_config_default(&cfg);
        cfg.initial_size = size;
        cfg.auto_resize = 0;
        check(dyc_create(&cfg, &t_), "hashAPI::hashAPI");
        check(dyc_pool_reserve(cfg.device, kPoolBytes), "hashAPI::hashAPI");
    }
    hashAPI(TYPE size, const dyc_config &cfg_in) {
        dyc_config cfg = cfg_in;
        cfg.initial_size = size;
        check(dyc_create(&cfg, &t_), "hashAPI::hashAPI");
        check(dyc_pool_reserve(cfg.device, kPoolBytes), "hashAPI::hashAPI");
    }
    static constexpr uint64_t kPoolBytes = 4ull << 30;
    ~hashAPI() {
        if (d_pool_k_) cudaFree(d_pool_k_);
        if (d_pool_v_) cudaFree(d_pool_v_);
        if (d_check_) cudaFree(d_check_);
        dyc_destroy(t_);
    }
    hashAPI(const hashAPI &) = delete;
    hashAPI &operator=(const hashAPI &) = delete;

    // api.cpp:184-265
    void hash_insert(TYPE *k, TYPE *v, TYPE size) {
        check(dyc_insert_host(t_, k, v, size, 0), "hashAPI::hash_insert");
    }
    // api.cpp:267-285: ans[i] = value of k[i], 0 on a miss
    void hash_search(TYPE *k, TYPE *ans, TYPE size) {
        check(dyc_find_host(t_, k, ans, nullptr, size), "hashAPI::hash_search");
    }
    // api.cpp:289-303
    uint64_t hash_delete(TYPE *k, TYPE *ans, TYPE size) {
        uint64_t n = 0;
        check(dyc_erase_host(t_, k, size, nullptr, &n), "hashAPI::hash_delete");
        if (ans) std::memset(ans, 0, sizeof(TYPE) * size);
        return n;
    }

    // api.cpp:309-344: one device copy of the whole pool, BATCH_SIZE slices
    bool set_data_to_gpu(TYPE *key, TYPE *value, TYPE size) {
        if ((uint64_t)size > (1024ull * 1024 * 1024) / (2 * sizeof(TYPE)))
            throw std::invalid_argument("set data error size of kv out of 2G");
        cuda(cudaMalloc(&d_pool_k_, sizeof(TYPE) * size), "cudaMalloc");
        cuda(cudaMalloc(&d_pool_v_, sizeof(TYPE) * size), "cudaMalloc");
        cuda(cudaMalloc(&d_check_, sizeof(TYPE) * BATCH_SIZE), "cudaMalloc");
        cuda(cudaMemcpy(d_pool_k_, key, sizeof(TYPE) * size, cudaMemcpyHostToDevice), "cudaMemcpy");
        cuda(cudaMemcpy(d_pool_v_, value, sizeof(TYPE) * size, cudaMemcpyHostToDevice), "cudaMemcpy");
        pool_size_ = size;
        return true;
    }
    void batch_reset() {  // api.cpp:346-351
        batch_num_to_op_ = batch_del_num_to_op_ = batch_search_num_to_op_ = 0;
    }
    // api.cpp:353-432: upsize while the projected size exceeds 0.8 capacity
    void hash_insert_batch() {
        if (batch_num_to_op_ >= BATCH_NUM) throw std::out_of_range("batch_num_to_op >= BATCH_NUM");
        const TYPE n = slice(batch_num_to_op_);
        while ((double)(num_size() + n) > kUpperBound * (double)table_size()) resize_up();
        check(dyc_insert(t_, d_pool_k_ + (size_t)batch_num_to_op_ * BATCH_SIZE,
                         d_pool_v_ + (size_t)batch_num_to_op_ * BATCH_SIZE, n,
                         DYC_FLAG_NO_RESIZE, nullptr),
              "hashAPI::hash_insert_batch");
        ++batch_num_to_op_;
    }
    // api.cpp:435-459 (results stay on the device, like the reference)
    void hash_search_batch() {
        if (batch_search_num_to_op_ >= BATCH_NUM) throw std::out_of_range("batch_search_num_to_op >= BATCH_NUM");
        const TYPE n = slice(batch_search_num_to_op_);
        check(dyc_find(t_, d_pool_k_ + (size_t)batch_search_num_to_op_ * BATCH_SIZE, d_check_,
                       nullptr, n, nullptr),
              "hashAPI::hash_search_batch");
        cuda(cudaStreamSynchronize(nullptr), "cudaStreamSynchronize");
        ++batch_search_num_to_op_;
    }
    // api.cpp:462-506: one downsize when below 0.5 capacity and above the guard
    void hash_delete_batch() {
        if (batch_del_num_to_op_ >= BATCH_NUM) throw std::out_of_range("batch_del_num_to_op >= BATCH_NUM");
        const TYPE n = slice(batch_del_num_to_op_);
        check(dyc_erase(t_, d_pool_k_ + (size_t)batch_del_num_to_op_ * BATCH_SIZE, n, nullptr,
                        nullptr, DYC_FLAG_NO_RESIZE, nullptr),
              "hashAPI::hash_delete_batch");
        ++batch_del_num_to_op_;
        if ((double)num_size() < kLowerBound * (double)table_size() &&
            (double)table_size() > kMinDownsizeCapacity)
            resize_low();
    }

    // api.cpp:112-141 and :143-173
    void resize_up() { check(dyc_resize_up(t_, nullptr), "hashAPI::resize_up"); }
    void resize_low() { check(dyc_resize_down(t_, nullptr), "hashAPI::resize_low"); }

    // hashAPI::num_size / table_size
    uint64_t num_size() const {
        uint64_t v = 0;
        check(dyc_size(t_, &v), "dyc_size");
        return v;
    }
    uint64_t table_size() const {
        uint64_t v = 0;
        check(dyc_capacity(t_, &v), "dyc_capacity");
        return v;
    }
    dyc_table *handle() const { return t_; }

  private:
    static void cuda(cudaError_t e, const char *what) {
        if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
    TYPE slice(int i) const {
        const uint64_t lo = (uint64_t)i * BATCH_SIZE;
        if (lo >= pool_size_) throw std::out_of_range("batch beyond the data set by set_data_to_gpu");
        const uint64_t n = pool_size_ - lo;
        return (TYPE)(n < (uint64_t)BATCH_SIZE ? n : BATCH_SIZE);
    }
    dyc_table *t_ = nullptr;
    TYPE *d_pool_k_ = nullptr, *d_pool_v_ = nullptr, *d_check_ = nullptr;
    uint64_t pool_size_ = 0;
    int batch_num_to_op_ = 0, batch_del_num_to_op_ = 0, batch_search_num_to_op_ = 0;
};

}  // namespace dycuckoo
