// noalloc.cu -- quids_gpu_rule_children_noalloc: the children enumeration of
// quids_gpu_rule_children for callers that cannot allocate device memory.
//
// The scratch the enumeration needs (per-parent child counts, the child
// offset scan with its look-back tiles, a few counters) lives in one
// file-scope static device array.  Every GPU that loads this library holds
// that array until the process exits.  Host code cannot use the array's name
// as a device address (it names a host-side stand-in), so every call looks
// the address up with cudaGetSymbolAddress on the current device, which must
// be the device of the caller's stream (a call synchronises its stream, so it
// is never part of a stream capture, and an address looked up per call stays
// valid across a cudaDeviceReset that reloads the module).  All calls on a
// device share the array: the parts that must start at zero are cleared at
// every call, and calls whose work overlaps on the GPU (e.g. issued on two
// streams at once) race on it.
#include <cmath>
#include <complex>
#include <cstdint>

#include "engine.cuh"
#include "rules_qc.cuh"
#include "rules_qcgd.cuh"

using namespace qd;
using namespace qd::engine;

namespace {

constexpr size_t round256(size_t v) { return (v + 255) / 256 * 256; }

constexpr uint64_t kMaxParents = QUIDS_NOALLOC_MAX_PARENTS;
constexpr uint64_t kMaxTiles = (kMaxParents + prim::kTile - 1) / prim::kTile;
// layout of the array: counters | look-back tiles | child counts | offsets
constexpr size_t kWordsOff = 0;  // u64: [0] parents, [1] children, [2] max child size, [3] status
constexpr size_t kLookbackOff = 256;
constexpr size_t kNchildOff = round256(kLookbackOff + (kMaxTiles + 2) * sizeof(uint64_t));
constexpr size_t kCbeginOff = round256(kNchildOff + kMaxParents * sizeof(uint32_t));
constexpr size_t kScratchBytes = round256(kCbeginOff + (kMaxParents + 1) * sizeof(uint64_t));
static_assert(kScratchBytes == QUIDS_NOALLOC_SCRATCH_BYTES, "header constant out of date");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// device address of the static scratch on the current device, which must be
// the device of `stream` (the null, legacy and per-thread default streams
// are the current device's)
int scratch_on_current_device(cudaStream_t stream, unsigned char **out, int *device) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return QUIDS_ERR_NO_DEVICE;
    }
    if (stream && stream != cudaStreamLegacy && stream != cudaStreamPerThread) {
        int sdev = -1;
        if (cudaStreamGetDevice(stream, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return QUIDS_ERR_BAD_ARG;
        }
        if (sdev != dev) return QUIDS_ERR_BAD_ARG;
    }
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
        cudaGetLastError();
        return QUIDS_ERR_CUDA;
    }
    *out = (unsigned char *)p;
    *device = dev;
    return QUIDS_OK;
}

qcgd::factors factors_of(const quids_gpu_rule_params *p) {
    std::complex<double> d = std::polar(std::sin(p->theta), p->phi);
    std::complex<double> dn = std::polar(std::cos(p->theta), p->xi);
    std::complex<double> ndnc = -std::conj(dn);
    return {{d.real(), d.imag()}, {d.real(), -d.imag()}, {dn.real(), dn.imag()}, {ndnc.real(), ndnc.imag()}};
}

template <class F>
int with_rule(int kind, const quids_gpu_rule_params *p, F &&f) {
    switch (kind) {
    case QUIDS_RULE_HADAMARD: return f(rules::hadamard{p->bit, 1 / std::sqrt(2)});
    case QUIDS_RULE_QCGD_ERASE_CREATE: return f(qcgd::erase_create{factors_of(p)});
    case QUIDS_RULE_QCGD_COIN: return f(qcgd::coin{factors_of(p)});
    case QUIDS_RULE_QCGD_SPLIT_MERGE: return f(qcgd::split_merge{factors_of(p)});
    }
    return QUIDS_ERR_BAD_ARG;
}

unsigned grid_of(int sms, uint64_t n) {
    uint64_t g = (n + prim::kThreads - 1) / prim::kThreads, cap = (uint64_t)sms * 8;
    return (unsigned)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

extern "C" int quids_gpu_rule_children_noalloc(void *stream, uint64_t num_object, const uint8_t *d_objects,
                                               const uint64_t *d_begin, const uint32_t *d_size,
                                               const double *d_magnitude, int rule_kind,
                                               const quids_gpu_rule_params *rule, uint64_t capacity,
                                               uint64_t *num_children, uint64_t *stride, uint8_t *d_child_bytes,
                                               uint64_t *d_hash, uint32_t *d_child_size,
                                               double *d_child_magnitude) {
    if (!rule || !num_children || !stride) return QUIDS_ERR_BAD_ARG;
    if (num_object > kMaxParents) return QUIDS_ERR_NOALLOC_LIMIT;
    if (num_object && (!d_objects || !d_begin || !d_size || !d_magnitude)) return QUIDS_ERR_BAD_ARG;
    if (rule_kind < QUIDS_RULE_HADAMARD || rule_kind > QUIDS_RULE_QCGD_SPLIT_MERGE) return QUIDS_ERR_BAD_ARG;
    unsigned char *base = nullptr;
    int dev = 0;
    QD_TRY(scratch_on_current_device((cudaStream_t)stream, &base, &dev));
    if (num_object == 0) {
        *num_children = 0;
        *stride = 8;
        return QUIDS_OK;
    }
    int sms = 0;
    QD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t *words = (uint64_t *)(base + kWordsOff);
    uint64_t *lbws = (uint64_t *)(base + kLookbackOff);
    uint32_t *nchild = (uint32_t *)(base + kNchildOff);
    uint64_t *cbegin = (uint64_t *)(base + kCbeginOff);
    const uint64_t tiles = (num_object + prim::kTile - 1) / prim::kTile;

    // the array keeps the previous call's contents: clear what must start at zero
    QD_CUDA(cudaMemsetAsync(words, 0, 256, s));
    QD_CUDA(cudaMemsetAsync(lbws, 0, (tiles + 2) * sizeof(uint64_t), s));
    k_set_word<<<1, 1, 0, s>>>(words + 0, num_object);
    QD_CUDA(cudaGetLastError());

    prim::lookback lb;
    lb.status = lbws + 1;
    lb.counter = (uint32_t *)lbws;
    lb.err = (int *)(words + 3);
    unsigned scan_grid = (unsigned)(tiles < (uint64_t)sms * 4 ? tiles : (uint64_t)sms * 4);
    int rc = with_rule(rule_kind, rule, [&](auto r) {
        k_num_child<<<grid_of(sms, num_object), prim::kThreads, 0, s>>>(
            single_rule<decltype(r)>{r}, (const char *)d_objects, d_begin, d_size, num_object, nchild, (unsigned long long *)(words + 2),
            (int *)(words + 3));
        prim::k_scan_excl<<<scan_grid, prim::kThreads, 0, s>>>(scan_nchild{nchild, nullptr}, words + 0, cbegin,
                                                               words + 1, lb);
        return cuda_status(cudaGetLastError());
    });
    if (rc) return rc;
    uint64_t h[4] = {0, 0, 0, 0};
    QD_CUDA(cudaMemcpyAsync(h, words, sizeof(h), cudaMemcpyDeviceToHost, s));
    QD_CUDA(cudaStreamSynchronize(s));
    if ((int)(int64_t)h[3]) return (int)(int64_t)h[3];
    const uint64_t nc = h[1];
    const uint64_t str = (h[2] + 7) / 8 * 8 + 8;
    *num_children = nc;
    *stride = str;
    if (!d_child_bytes || nc == 0) return QUIDS_OK;
    if (capacity < nc || !d_hash || !d_child_size || !d_child_magnitude) return QUIDS_ERR_BAD_ARG;

    QD_CUDA(cudaMemsetAsync(d_child_bytes, 0, nc * str, s));
    parents_view pv{(const char *)d_objects, d_begin, d_size, (const double2 *)d_magnitude, cbegin, nullptr,
                    num_object};
    rc = with_rule(rule_kind, rule, [&](auto r) {
        k_children<<<grid_of(sms, nc), prim::kThreads, 0, s>>>(r, pv, nc, str, (char *)d_child_bytes, d_hash,
                                                             d_child_size, (double2 *)d_child_magnitude);
        return cuda_status(cudaGetLastError());
    });
    if (rc) return rc;
    QD_CUDA(cudaStreamSynchronize(s));
    return QUIDS_OK;
}
