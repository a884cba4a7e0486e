// csc_cache.cpp - the reference's binary CSC matrix cache files (host only).
//
// The reference's molecule benchmarks store a generated FCI Hamiltonian as
// one file (write_ch4_matrix_cache / read_ch4_matrix_cache,
// IPT_C_GPU/test/sparse/CH4/benchmark_ch4_sto6g_fci_15876_ipt.cu:1015-1121;
// the same layout under other magics in the H2O, NH3 and generic benchmarks;
// field offsets also in results/sparse/CH4_K30_debug/inspect_csc_bin.py:7-57):
//
//   0   char[8]  magic "IPT" + molecule tag + "C1" (IPTCH4C1, IPTH2OC1, IPTNH3C1, IPTGENC1)
//   8   uint32   version (1)
//   12  int32    n
//   16  int32    nnz          (4 zero bytes follow: the next field is 8-aligned)
//   24  double   ||H||_inf
//   32  int32    norb, nelec, neleca, nelecb, na, nb   (56 bytes in all)
//   56  int32    col_ptr[n + 1], int32 row_ind[nnz], double values[nnz], double diagonal[n]
//
// little-endian, as written by the reference on x86-64 and read back here on
// x86-64 and aarch64 alike.  Loading such a file lets the solver run on the
// reference's own matrices where the files exist.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <cstdint>
#include <vector>

#include "../../include/ipt_block.h"
#include "prep.h"

namespace {

constexpr size_t kHeaderBytes = 56;

void put_u32(unsigned char *p, uint32_t v)
{
    for (int i = 0; i < 4; ++i) p[i] = (unsigned char)(v >> (8 * i));
}

uint32_t get_u32(const unsigned char *p)
{
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)p[i] << (8 * i);
    return v;
}

void put_f64(unsigned char *p, double d)
{
    uint64_t v;
    memcpy(&v, &d, sizeof(v));
    for (int i = 0; i < 8; ++i) p[i] = (unsigned char)(v >> (8 * i));
}

double get_f64(const unsigned char *p)
{
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p[i] << (8 * i);
    double d;
    memcpy(&d, &v, sizeof(d));
    return d;
}

bool magic_ok(const unsigned char *m)
{
    return m[0] == 'I' && m[1] == 'P' && m[2] == 'T' && m[6] == 'C' && m[7] == '1';
}

bool read_header(FILE *f, IPTCscCacheInfo *info)
{
    unsigned char h[kHeaderBytes];
    if (fread(h, 1, kHeaderBytes, f) != kHeaderBytes || !magic_ok(h)) return false;
    memset(info, 0, sizeof(*info));
    memcpy(info->magic, h, 8);
    info->magic[8] = '\0';
    info->version = (int)get_u32(h + 8);
    info->n = (int32_t)get_u32(h + 12);
    info->nnz = (int32_t)get_u32(h + 16);
    info->matrix_inf_norm = get_f64(h + 24);
    int32_t *dst[6] = {&info->norb, &info->nelec, &info->neleca, &info->nelecb, &info->na,
                       &info->nb};
    for (int i = 0; i < 6; ++i) *dst[i] = (int32_t)get_u32(h + 32 + 4 * i);
    return info->version == 1 && info->n > 0 && info->nnz >= 0;
}

// little-endian arrays, element by element (no host byte-order assumption)
template <typename T>
bool read_array(FILE *f, T *out, size_t count)
{
    std::vector<unsigned char> buf(count * sizeof(T));
    if (count > 0 && fread(buf.data(), 1, buf.size(), f) != buf.size()) return false;
    for (size_t i = 0; i < count; ++i) {
        uint64_t v = 0;
        for (size_t b = 0; b < sizeof(T); ++b) v |= (uint64_t)buf[i * sizeof(T) + b] << (8 * b);
        if (sizeof(T) == 4) {
            const uint32_t w = (uint32_t)v;
            memcpy(&out[i], &w, sizeof(T));
        } else {
            memcpy(&out[i], &v, sizeof(T));
        }
    }
    return true;
}

template <typename T>
bool write_array(FILE *f, const T *in, size_t count)
{
    std::vector<unsigned char> buf(count * sizeof(T));
    for (size_t i = 0; i < count; ++i) {
        uint64_t v = 0;
        if (sizeof(T) == 4) {
            uint32_t w;
            memcpy(&w, &in[i], sizeof(T));
            v = w;
        } else {
            memcpy(&v, &in[i], sizeof(T));
        }
        for (size_t b = 0; b < sizeof(T); ++b) buf[i * sizeof(T) + b] = (unsigned char)(v >> (8 * b));
    }
    return count == 0 || fwrite(buf.data(), 1, buf.size(), f) == buf.size();
}

}  // namespace

#define IPT_API extern "C" __attribute__((visibility("default")))

IPT_API int ipt_block_csc_cache_info(const char *path, IPTCscCacheInfo *info)
{
    if (path == nullptr || path[0] == '\0' || info == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    FILE *f = fopen(path, "rb");
    if (f == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    const bool ok = read_header(f, info);
    fclose(f);
    return ok ? IPT_CUDA_SUCCESS : IPT_CUDA_INVALID_ARGUMENT;
}

IPT_API int ipt_block_csc_cache_read(const char *path, int *col_ptr, int *row_ind, double *values,
                                     double *diagonal, int n_capacity, int nnz_capacity,
                                     IPTCscCacheInfo *info)
{
    if (path == nullptr || path[0] == '\0' || info == nullptr || col_ptr == nullptr ||
        values == nullptr || row_ind == nullptr || diagonal == nullptr) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    FILE *f = fopen(path, "rb");
    if (f == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    bool ok = read_header(f, info) && info->n <= n_capacity && info->nnz <= nnz_capacity;
    ok = ok && read_array(f, col_ptr, (size_t)info->n + 1U) &&
         read_array(f, row_ind, (size_t)info->nnz) && read_array(f, values, (size_t)info->nnz) &&
         read_array(f, diagonal, (size_t)info->n);
    fclose(f);
    // the reference rejects a file whose arrays are not a valid CSC or whose
    // norm is negative or not finite (benchmark_ch4_...cu:1107-1113)
    if (!ok || !iptgb::validate_csc(col_ptr, row_ind, info->n, info->nnz) ||
        !isfinite(info->matrix_inf_norm) || info->matrix_inf_norm < 0.0) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    return IPT_CUDA_SUCCESS;
}

IPT_API int ipt_block_csc_cache_write(const char *path, const IPTCscCacheInfo *info,
                                      const int *col_ptr, const int *row_ind,
                                      const double *values, const double *diagonal)
{
    if (path == nullptr || path[0] == '\0' || info == nullptr || col_ptr == nullptr ||
        diagonal == nullptr || info->n <= 0 || info->nnz < 0 ||
        (info->nnz > 0 && (row_ind == nullptr || values == nullptr)) ||
        !magic_ok((const unsigned char *)info->magic) ||
        !iptgb::validate_csc(col_ptr, row_ind, info->n, info->nnz)) {
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    unsigned char h[kHeaderBytes] = {};
    memcpy(h, info->magic, 8);
    put_u32(h + 8, 1u);
    put_u32(h + 12, (uint32_t)info->n);
    put_u32(h + 16, (uint32_t)info->nnz);
    put_f64(h + 24, info->matrix_inf_norm);
    const int32_t src[6] = {info->norb, info->nelec, info->neleca, info->nelecb, info->na, info->nb};
    for (int i = 0; i < 6; ++i) put_u32(h + 32 + 4 * i, (uint32_t)src[i]);
    // written to path.tmp, then renamed over path (as the reference does)
    std::vector<char> tmp(strlen(path) + 5);
    snprintf(tmp.data(), tmp.size(), "%s.tmp", path);
    FILE *f = fopen(tmp.data(), "wb");
    if (f == nullptr) return IPT_CUDA_INVALID_ARGUMENT;
    bool ok = fwrite(h, 1, kHeaderBytes, f) == kHeaderBytes &&
              write_array(f, col_ptr, (size_t)info->n + 1U) &&
              write_array(f, row_ind, (size_t)info->nnz) &&
              write_array(f, values, (size_t)info->nnz) &&
              write_array(f, diagonal, (size_t)info->n) && fflush(f) == 0;
    if (fclose(f) != 0) ok = false;
    if (!ok || rename(tmp.data(), path) != 0) {
        remove(tmp.data());
        return IPT_CUDA_INVALID_ARGUMENT;
    }
    return IPT_CUDA_SUCCESS;
}
