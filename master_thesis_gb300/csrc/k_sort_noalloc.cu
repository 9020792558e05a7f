// k_sort_noalloc.cu - the radix sort of k_sort.cu for callers that cannot allocate device memory.
//
// The scratch lives in one file-scope device array sized for TECTO_SORT_NOALLOC_MAX_PAIRS pairs
// of 32-bit keys: the sort's histograms and look-back status, plus one key/value ping-pong half.
// The caller's output buffers serve as the other half (the last pass always writes them).
// Host code cannot use the array's name as a device address, so its address is looked up with
// cudaGetSymbolAddress once per device, with that device current, on the first call there.
#include <mutex>
#include <unordered_map>

#include "tecto_internal.cuh"

namespace tecto {
namespace {

constexpr size_t kMaxPairs = TECTO_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }
// sort_scratch_bytes(kMaxPairs, 32, 8): histograms, look-back status (4 passes), counters, error word
constexpr size_t kSortPart = a256((size_t)kMaxSortPasses * 256 * 4) +
                             a256((size_t)kMaxSortPasses * ((kMaxPairs + kSortTile - 1) / kSortTile) * 256 * 4) +
                             a256((size_t)kMaxSortPasses * 4) + a256(4);
constexpr size_t kHalf = a256(kMaxPairs * sizeof(uint32_t));
constexpr size_t kScratchBytes = kSortPart + 2 * kHalf;

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

std::mutex g_mu;
std::unordered_map<int, void *> g_addr;  // device ordinal -> address of g_sort_scratch there

// Device address of g_sort_scratch on the current device (looked up once per device; the address
// stays valid for the life of the device's context, so cudaDeviceReset is not supported while the
// library is in use).
int scratch_address(void **out)
{
    int dev = 0;
    TECTO_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_addr.find(dev);
    if (it == g_addr.end()) {
        void *p = nullptr;
        TECTO_CUDA(cudaGetSymbolAddress(&p, g_sort_scratch));
        it = g_addr.emplace(dev, p).first;
    }
    *out = it->second;
    return TECTO_OK;
}

bool overlaps(const void *a, const void *b, size_t bytes)
{
    const char *x = (const char *)a, *y = (const char *)b;
    return x < y + bytes && y < x + bytes;
}

}  // namespace
}  // namespace tecto

extern "C" int tecto_sort_pairs_noalloc(const uint32_t *keys_in, const uint32_t *vals_in,
                                        uint32_t *keys_out, uint32_t *vals_out, size_t n, int key_bits,
                                        tecto_stream_t stream)
{
    using namespace tecto;
    if (n == 0) return TECTO_OK;
    if (!keys_in || !vals_in || !keys_out || !vals_out || key_bits < 1 || key_bits > 32) {
        set_error("tecto_sort_pairs_noalloc: invalid argument");
        return TECTO_ERR_INVALID;
    }
    if (n > kMaxPairs) {
        set_error("tecto_sort_pairs_noalloc: n exceeds TECTO_SORT_NOALLOC_MAX_PAIRS (1048576 pairs); "
                  "use tecto_sort_pairs with caller-provided scratch");
        return TECTO_ERR_INVALID;
    }
    const size_t bytes = n * sizeof(uint32_t);
    if (overlaps(keys_out, keys_in, bytes) || overlaps(keys_out, vals_in, bytes) ||
        overlaps(vals_out, keys_in, bytes) || overlaps(vals_out, vals_in, bytes) ||
        overlaps(keys_out, vals_out, bytes)) {
        set_error("tecto_sort_pairs_noalloc: outputs must not alias the inputs or each other");
        return TECTO_ERR_INVALID;
    }
    void *base = nullptr;
    int rc = scratch_address(&base);
    if (rc != TECTO_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    SortScratch scr{};
    sort_scratch_carve(base, n, key_bits, 8, &scr);  // fits: sized for the maximum n and 4 passes
    char *half = (char *)base + kSortPart;
    const int passes = sort_passes_for(key_bits, 8);
    const int last = (passes - 1) & 1;  // the half the final pass writes: the caller's outputs
    SortArgs a{};
    a.keys_in = keys_in;
    a.vals_in = vals_in;
    a.keys[last] = keys_out;
    a.vals[last] = vals_out;
    a.keys[last ^ 1] = (uint32_t *)half;
    a.vals[last ^ 1] = (uint32_t *)(half + kHalf);
    a.n = n;
    a.key_bits = key_bits;
    TECTO_CUDA(cudaMemsetAsync(scr.error, 0, 4, st));  // the array keeps the previous call's flag
    int result_half = -1;
    rc = run_sort(a, scr, st, &result_half);
    if (rc != TECTO_OK) return rc;
    if (result_half != last) {
        set_error("tecto_sort_pairs_noalloc: internal pass parity mismatch");
        return TECTO_ERR_INVALID;
    }
    uint32_t err = 0;
    TECTO_CUDA(cudaMemcpyAsync(&err, scr.error, 4, cudaMemcpyDeviceToHost, st));
    TECTO_CUDA(cudaStreamSynchronize(st));
    if (err) {
        set_error("tecto_sort_pairs_noalloc: look-back wait gave up");
        return TECTO_ERR_DEVICE_TIMEOUT;
    }
    return TECTO_OK;
}
