// tecto_export.cu - headless output of a world: the reference's two image exports as PNG files,
// and raw snapshots of the complete world state (checkpoint and resume).
//
// Images follow src/cuda_compute/texture_save.cu:
//  - heights: saveFloatCudaTextureToDiskAsGray16 (:255-294, convertFloatToGray16Kernel :80-96),
//    norm = clamp((v - min) / (max - min), 0, 1), value = (uint16) (norm * 65535), 16-bit grayscale;
//    the reference passes minUpliftClamp / maxUpliftClamp as the range (plate_tectonic_sim.cu:635);
//  - plate ids: saveGrayscale8BitCudaTextureToDiskAsRgb (:222-252, convertGrayscaleToRgbKernel
//    :10-78), an HSV colour per id (id 255: the background colour).  Only 256 ids exist, so the
//    colours form a 256-entry palette computed once on the host.
// The reference writes PNG through libpng; this file has its own minimal encoder (zlib stream of
// stored deflate blocks, CRC-32 and Adler-32 as in RFC 1950/1951 and the PNG specification), so
// the files differ in bytes but decode to the same pixels.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tecto_internal.cuh"

namespace tecto {
namespace {

__global__ void k_gray16(const float *h, uint16_t *out, size_t n, float minv, float maxv)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        float norm = (h[i] - minv) / (maxv - minv);
        norm = fminf(fmaxf(norm, 0.0f), 1.0f);
        out[i] = (uint16_t)(norm * 65535.0f);
    }
}

struct Palette {
    uint8_t rgb[256 * 3];
};

// convertGrayscaleToRgbKernel as a palette lookup (the colour depends on the id alone).
__global__ void k_ids_rgb(const uint8_t *ids, uint8_t *out, size_t n, const Palette pal)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint8_t *c = pal.rgb + 3 * ids[i];
        out[3 * i] = c[0];
        out[3 * i + 1] = c[1];
        out[3 * i + 2] = c[2];
    }
}

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init()
{
    if (crc_ready) return;
    for (uint32_t n = 0; n < 256; ++n) {
        uint32_t c = n;
        for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = true;
}

uint32_t crc32(uint32_t crc, const uint8_t *p, size_t n)
{
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = crc_table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}

void put32(std::vector<uint8_t> &v, uint32_t x)
{
    v.push_back((uint8_t)(x >> 24));
    v.push_back((uint8_t)(x >> 16));
    v.push_back((uint8_t)(x >> 8));
    v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t> &png, const char *type, const std::vector<uint8_t> &data)
{
    put32(png, (uint32_t)data.size());
    const size_t at = png.size();
    png.insert(png.end(), type, type + 4);
    png.insert(png.end(), data.begin(), data.end());
    put32(png, crc32(0, png.data() + at, data.size() + 4));
}

// kind: 0 gray16 (pixels: uint16 per pixel, host order), 1 rgb8 (3 bytes per pixel), 2 gray8.
// srgb: add the sRGB chunk (perceptual intent) the reference's 16-bit export writes
// (texture_save.cu:187).
int encode_png(const void *pixels, int w, int h, int kind, std::vector<uint8_t> &png, bool srgb = false)
{
    if (!pixels || w < 1 || h < 1 || kind < 0 || kind > 2) return TECTO_ERR_INVALID;
    crc_init();
    const int bpp = kind == 0 ? 2 : kind == 1 ? 3 : 1;
    const size_t row = (size_t)w * bpp;
    // raw scanlines, filter type 0, samples big-endian
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * (size_t)h);
    const uint8_t *src = (const uint8_t *)pixels;
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        if (kind == 0) {
            const uint16_t *p = (const uint16_t *)pixels + (size_t)y * w;
            for (int x = 0; x < w; ++x) {
                raw.push_back((uint8_t)(p[x] >> 8));
                raw.push_back((uint8_t)p[x]);
            }
        } else {
            raw.insert(raw.end(), src + (size_t)y * row, src + (size_t)(y + 1) * row);
        }
    }
    // zlib stream of stored deflate blocks
    std::vector<uint8_t> z;
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    size_t pos = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)len);
        z.push_back((uint8_t)(len >> 8));
        z.push_back((uint8_t)~len);
        z.push_back((uint8_t)(~len >> 8));
        z.insert(z.end(), raw.begin() + (long)pos, raw.begin() + (long)(pos + len));
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(z, (b << 16) | a);
    png.clear();
    const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a};
    png.insert(png.end(), sig, sig + 8);
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)w);
    put32(ihdr, (uint32_t)h);
    ihdr.push_back(kind == 0 ? 16 : 8);           // bit depth
    ihdr.push_back(kind == 1 ? 2 : 0);            // colour type: truecolour or grayscale
    ihdr.push_back(0);                            // deflate
    ihdr.push_back(0);                            // adaptive filtering
    ihdr.push_back(0);                            // no interlace
    chunk(png, "IHDR", ihdr);
    if (srgb) chunk(png, "sRGB", {0});
    chunk(png, "IDAT", z);
    chunk(png, "IEND", {});
    return TECTO_OK;
}

// convertGrayscaleToRgbKernel's colour of one plate id (texture_save.cu:16-70)
void plate_colour(int val, uint8_t *rgb)
{
    if (val == 255) {
        rgb[0] = 230;
        rgb[1] = 235;
        rgb[2] = 240;
        return;
    }
    const float h = 0.125f * (float)(val % 8) + (float)val / 8.0f / 256.0f;  // float division
    const float s = 0.5f + 0.5f * sinf((float)val * 0.1f);
    const float v = 0.5f + 0.5f * cosf((float)val * 0.1f);
    const float c = v * s;
    const float x = c * (1.0f - fabsf(fmodf(h * 6.0f, 2.0f) - 1.0f));
    const float m = v - c;
    float r, g, b;
    const double hd = h;
    if (hd >= 0.0 && hd < 1.0 / 6.0) { r = c; g = x; b = 0.0f; }
    else if (hd >= 1.0 / 6.0 && hd < 2.0 / 6.0) { r = x; g = c; b = 0.0f; }
    else if (hd >= 2.0 / 6.0 && hd < 3.0 / 6.0) { r = 0.0f; g = c; b = x; }
    else if (hd >= 3.0 / 6.0 && hd < 4.0 / 6.0) { r = 0.0f; g = x; b = c; }
    else if (hd >= 4.0 / 6.0 && hd < 5.0 / 6.0) { r = x; g = 0.0f; b = c; }
    else { r = c; g = 0.0f; b = x; }
    rgb[0] = (uint8_t)std::lround((r + m) * 255.0f);
    rgb[1] = (uint8_t)std::lround((g + m) * 255.0f);
    rgb[2] = (uint8_t)std::lround((b + m) * 255.0f);
}

int write_file(const char *path, const void *data, size_t n)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        set_error(std::string("cannot open ") + path + " for writing");
        return TECTO_ERR_INVALID;
    }
    const size_t wrote = std::fwrite(data, 1, n, f);
    const int closed = std::fclose(f);
    if (wrote != n || closed != 0) {
        set_error(std::string("cannot write ") + path);
        return TECTO_ERR_INVALID;
    }
    return TECTO_OK;
}

// ---- snapshots ----------------------------------------------------------------------------------
// File: SnapHeader, tecto_settings, the fields of snap_fields() in that order, the 255 plate records,
// the 255 plate dynamics records, then the asthenosphere pressure texture (pw x ph floats), all in
// the host's byte order.

constexpr char kMagic[8] = {'T', 'E', 'C', 'T', 'O', 'S', 'N', '2'};

struct SnapHeader {
    char magic[8];
    uint32_t header_bytes, settings_bytes;
    int32_t width, height;
    uint32_t seed, iteration;
    uint64_t cells;
    int32_t pw, ph;  // asthenosphere pressure texture, 0 x 0 when there is none
};

struct SnapField {
    int field;
    size_t bytes;
};

std::vector<SnapField> snap_fields(size_t N)
{
    return {{TECTO_FIELD_HEIGHT, N * 4},      {TECTO_FIELD_WATER, N * 4},        {TECTO_FIELD_SEDIMENT, N * 4},
            {TECTO_FIELD_FLUX, N * 16},       {TECTO_FIELD_PLATE_ID, N},         {TECTO_FIELD_LABELS, N * 4},
            {TECTO_FIELD_TYPE_BITMAP, kPairs}, {TECTO_FIELD_DIV_BITMAP, (size_t)kDivWords * 4}};
}

}  // namespace
}  // namespace tecto

using namespace tecto;

extern "C" {

int tecto_png_encode(const void *pixels, int width, int height, int kind, void *out, size_t capacity,
                     size_t *written)
{
    std::vector<uint8_t> png;
    const int rc = encode_png(pixels, width, height, kind, png);
    if (rc != TECTO_OK) {
        set_error("tecto_png_encode: invalid argument");
        return rc;
    }
    if (written) *written = png.size();
    if (!out) return TECTO_OK;  // size query
    if (capacity < png.size()) {
        set_error("tecto_png_encode: output buffer too small");
        return TECTO_ERR_INVALID;
    }
    std::memcpy(out, png.data(), png.size());
    return TECTO_OK;
}

int tecto_plate_palette(uint8_t *rgb768)
{
    if (!rgb768) return TECTO_ERR_INVALID;
    for (int v = 0; v < 256; ++v) plate_colour(v, rgb768 + 3 * v);
    return TECTO_OK;
}

int tecto_world_export_png(tecto_world *w, int kind, const char *path, float min_value, float max_value,
                           tecto_stream_t stream)
{
    if (!w || !path || (kind != TECTO_EXPORT_HEIGHT_GRAY16 && kind != TECTO_EXPORT_PLATES_RGB)) {
        set_error("tecto_world_export_png: invalid argument");
        return TECTO_ERR_INVALID;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    const size_t N = w->N;
    std::vector<uint8_t> png;
    int rc;
    if (kind == TECTO_EXPORT_HEIGHT_GRAY16) {
        if (!(max_value > min_value)) {
            set_error("tecto_world_export_png: the height range is empty");
            return TECTO_ERR_INVALID;
        }
        void *dh = nullptr;
        size_t bytes = 0;
        if ((rc = tecto_world_field(w, TECTO_FIELD_HEIGHT, &dh, &bytes)) != TECTO_OK) return rc;
        uint16_t *d16 = nullptr;
        TECTO_CUDA(cudaMalloc(&d16, N * 2));
        const unsigned grid = (unsigned)std::min<size_t>((N + 255) / 256, 152 * 16);
        k_gray16<<<grid, 256, 0, st>>>((const float *)dh, d16, N, min_value, max_value);
        std::vector<uint16_t> g(N);
        cudaError_t e = cudaMemcpyAsync(g.data(), d16, N * 2, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(d16);
        if (e != cudaSuccess) return cuda_fail(e, "tecto_world_export_png");
        rc = encode_png(g.data(), w->W, w->H, 0, png, true);
    } else {
        void *dids = nullptr;
        size_t bytes = 0;
        if ((rc = tecto_world_field(w, TECTO_FIELD_PLATE_ID, &dids, &bytes)) != TECTO_OK) return rc;
        Palette pal;
        for (int v = 0; v < 256; ++v) plate_colour(v, pal.rgb + 3 * v);
        uint8_t *drgb = nullptr;
        TECTO_CUDA(cudaMalloc(&drgb, N * 3));
        const unsigned grid = (unsigned)std::min<size_t>((N + 255) / 256, 152 * 16);
        k_ids_rgb<<<grid, 256, 0, st>>>((const uint8_t *)dids, drgb, N, pal);
        std::vector<uint8_t> rgb(N * 3);
        cudaError_t e = cudaMemcpyAsync(rgb.data(), drgb, N * 3, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(drgb);
        if (e != cudaSuccess) return cuda_fail(e, "tecto_world_export_png");
        rc = encode_png(rgb.data(), w->W, w->H, 1, png);
    }
    if (rc != TECTO_OK) return rc;
    return write_file(path, png.data(), png.size());
}

int tecto_world_save_snapshot(tecto_world *w, const char *path, tecto_stream_t stream)
{
    if (!w || !path) return TECTO_ERR_INVALID;
    SnapHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.header_bytes = sizeof(SnapHeader);
    hd.settings_bytes = sizeof(tecto_settings);
    hd.width = w->W;
    hd.height = w->H;
    hd.seed = w->seed;
    hd.iteration = w->iteration;
    hd.cells = w->N;
    hd.pw = w->pw;
    hd.ph = w->ph;
    std::vector<uint8_t> buf(sizeof(hd) + sizeof(tecto_settings));
    std::memcpy(buf.data(), &hd, sizeof(hd));
    std::memcpy(buf.data() + sizeof(hd), &w->settings, sizeof(tecto_settings));
    int rc;
    for (const SnapField &f : snap_fields(w->N)) {
        const size_t at = buf.size();
        buf.resize(at + f.bytes);
        if ((rc = tecto_world_download(w, f.field, buf.data() + at, f.bytes, stream)) != TECTO_OK) return rc;
    }
    std::vector<tecto_plate> plates(kPlates);
    if ((rc = tecto_world_get_plates(w, plates.data(), kPlates, stream)) != TECTO_OK) return rc;
    size_t at = buf.size();
    buf.resize(at + plates.size() * sizeof(tecto_plate));
    std::memcpy(buf.data() + at, plates.data(), plates.size() * sizeof(tecto_plate));
    std::vector<tecto_plate_dynamics> dyn(kPlates);
    if ((rc = tecto_world_get_plate_dynamics(w, dyn.data(), kPlates, stream)) != TECTO_OK) return rc;
    at = buf.size();
    buf.resize(at + dyn.size() * sizeof(tecto_plate_dynamics));
    std::memcpy(buf.data() + at, dyn.data(), dyn.size() * sizeof(tecto_plate_dynamics));
    if (w->pressure) {
        at = buf.size();
        const size_t bytes = (size_t)w->pw * (size_t)w->ph * 4;
        buf.resize(at + bytes);
        TECTO_CUDA(cudaMemcpy(buf.data() + at, w->pressure, bytes, cudaMemcpyDeviceToHost));
    }
    return write_file(path, buf.data(), buf.size());
}

int tecto_snapshot_info(const char *path, int *width, int *height, tecto_settings *settings)
{
    if (!path) return TECTO_ERR_INVALID;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return TECTO_ERR_INVALID;
    }
    SnapHeader hd{};
    tecto_settings s{};
    const bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, kMagic, 8) == 0 &&
                    hd.header_bytes == sizeof(SnapHeader) && hd.settings_bytes == sizeof(tecto_settings) &&
                    std::fread(&s, sizeof(s), 1, f) == 1;
    std::fclose(f);
    if (!ok) {
        set_error(std::string(path) + " is not a snapshot of this engine version");
        return TECTO_ERR_INVALID;
    }
    if (width) *width = hd.width;
    if (height) *height = hd.height;
    if (settings) *settings = s;
    return TECTO_OK;
}

int tecto_world_load_snapshot(tecto_world *w, const char *path, tecto_stream_t stream)
{
    if (!w || !path) return TECTO_ERR_INVALID;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error(std::string("cannot open ") + path);
        return TECTO_ERR_INVALID;
    }
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    std::vector<uint8_t> buf(size > 0 ? (size_t)size : 0);
    const bool read = size > 0 && std::fread(buf.data(), 1, buf.size(), f) == buf.size();
    std::fclose(f);
    SnapHeader hd{};
    size_t need = sizeof(hd) + sizeof(tecto_settings) + kPlates * (sizeof(tecto_plate) + sizeof(tecto_plate_dynamics));
    if (read && buf.size() >= sizeof(hd)) std::memcpy(&hd, buf.data(), sizeof(hd));
    for (const SnapField &fl : snap_fields((size_t)hd.cells)) need += fl.bytes;
    if (hd.pw < 0 || hd.ph < 0 || (size_t)hd.pw * (size_t)hd.ph > ((size_t)1 << 30)) need = 0;
    else need += (size_t)hd.pw * (size_t)hd.ph * 4;
    if (!read || std::memcmp(hd.magic, kMagic, 8) != 0 || hd.header_bytes != sizeof(SnapHeader) ||
        hd.settings_bytes != sizeof(tecto_settings) || buf.size() != need) {
        set_error(std::string(path) + " is not a snapshot of this engine version");
        return TECTO_ERR_INVALID;
    }
    if (hd.width != w->W || hd.height != w->H) {
        set_error("tecto_world_load_snapshot: the snapshot's size differs from the world's");
        return TECTO_ERR_INVALID;
    }
    tecto_settings s;
    std::memcpy(&s, buf.data() + sizeof(hd), sizeof(s));
    int rc;
    if ((rc = tecto_world_set_settings(w, &s)) != TECTO_OK) return rc;
    size_t at = sizeof(hd) + sizeof(s);
    for (const SnapField &fl : snap_fields(w->N)) {
        if ((rc = tecto_world_upload(w, fl.field, buf.data() + at, fl.bytes, stream)) != TECTO_OK) return rc;
        at += fl.bytes;
    }
    if ((rc = tecto_world_set_plates(w, (const tecto_plate *)(buf.data() + at), kPlates, stream)) != TECTO_OK)
        return rc;
    at += kPlates * sizeof(tecto_plate);
    std::vector<tecto_plate_dynamics> dyn(kPlates);
    std::memcpy(dyn.data(), buf.data() + at, kPlates * sizeof(tecto_plate_dynamics));
    if ((rc = tecto_world_set_plate_dynamics(w, dyn.data(), kPlates, stream)) != TECTO_OK) return rc;
    at += kPlates * sizeof(tecto_plate_dynamics);
    std::vector<float> pressure((size_t)hd.pw * (size_t)hd.ph);
    if (!pressure.empty()) std::memcpy(pressure.data(), buf.data() + at, pressure.size() * 4);
    if ((rc = tecto_world_set_asthenosphere(w, pressure.empty() ? nullptr : pressure.data(), hd.pw, hd.ph,
                                            stream)) != TECTO_OK)
        return rc;
    if ((rc = tecto_world_set_iteration(w, hd.iteration)) != TECTO_OK) return rc;
    w->seed = hd.seed;
    TECTO_CUDA(cudaMemcpy(&w->dev.ctl->seed, &hd.seed, 4, cudaMemcpyHostToDevice));
    return TECTO_OK;
}

}  // extern "C"
