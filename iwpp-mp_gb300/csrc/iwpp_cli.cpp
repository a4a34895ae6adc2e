// iwpp_cli.cpp -- command-line front end with the reference's arguments,
// without OpenCV:
//
//   iwpp_cli <marker> <mask> <output> <usePGMLoader> [options]
//
// as IWPP MP DQ/src/main.cu:145-241: read marker and mask, clip the marker
// under the mask (the reference's clipImage launch, main.cu:223), time the
// reconstruction in milliseconds (printed as the reference prints it,
// main.cu:231-232), write the result.  The reference reads PGM with its own
// loader when usePGMLoader is 1 (main.cu:27-112) and anything OpenCV reads
// otherwise; here both read binary / ASCII PGM (8- and 16-bit), uncompressed
// TIFF and raw files, chosen by content / extension, and usePGMLoader is
// accepted for compatibility.  Output format by extension: .pgm, .tif /
// .tiff (uncompressed), anything else raw bytes.
//
// options: --conn 4|8 (default 4, the reference's), --variant
// mutex|double|unique|async|default, --raw WxH:u8|u16|i32 (how to read .raw
// inputs), --no-clip, --repeat N (time N runs from the same marker, report
// the median), --init-passes N, --solver 0|1|2, --tile-rows 32|64 (the
// iwpp_config fields; default: the library's defaults), --convert IN OUT
// (I/O only, no GPU: rewrite IN as OUT).
#include <algorithm>
#include <cctype>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "iwpp.h"

namespace {

struct Image {
    int w = 0, h = 0;
    int dtype = IWPP_U8;  // IWPP_U8 / U16 / I32
    std::vector<unsigned char> px;  // row-major, w * bpp bytes per row, host byte order
    size_t bpp() const { return dtype == IWPP_U8 ? 1 : dtype == IWPP_U16 ? 2 : 4; }
};

bool fail(const char* what, const std::string& path) {
    std::fprintf(stderr, "iwpp_cli: %s: %s\n", what, path.c_str());
    return false;
}

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)s[s.size() - n + i]) != suf[i]) return false;
    return true;
}

bool read_file(const std::string& path, std::vector<unsigned char>& out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    unsigned char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) out.insert(out.end(), buf, buf + n);
    std::fclose(f);
    return true;
}

// ---- PGM (P5 binary, P2 ASCII); 16-bit samples are big-endian in P5
bool pgm_token(const std::vector<unsigned char>& d, size_t& i, long& v) {
    for (;;) {
        while (i < d.size() && std::isspace(d[i])) ++i;
        if (i < d.size() && d[i] == '#') {
            while (i < d.size() && d[i] != '\n') ++i;
            continue;
        }
        break;
    }
    if (i >= d.size() || !std::isdigit(d[i])) return false;
    v = 0;
    while (i < d.size() && std::isdigit(d[i])) {
        v = v * 10 + (d[i] - '0');
        if (v > (1l << 30)) return false;
        ++i;
    }
    return true;
}

bool read_pgm(const std::string& path, const std::vector<unsigned char>& d, Image& im) {
    if (d.size() < 2 || d[0] != 'P' || (d[1] != '5' && d[1] != '2')) return fail("not a PGM file", path);
    size_t i = 2;
    long w, h, maxv;
    if (!pgm_token(d, i, w) || !pgm_token(d, i, h) || !pgm_token(d, i, maxv)) return fail("bad PGM header", path);
    if (w <= 0 || h <= 0 || maxv <= 0 || maxv > 65535) return fail("bad PGM dimensions", path);
    im.w = (int)w;
    im.h = (int)h;
    im.dtype = maxv > 255 ? IWPP_U16 : IWPP_U8;
    const size_t n = (size_t)w * h;
    im.px.assign(n * im.bpp(), 0);
    if (d[1] == '5') {
        ++i;  // the single whitespace after maxval
        if (d.size() < i + n * im.bpp()) return fail("PGM data too short", path);
        if (im.dtype == IWPP_U8) {
            std::memcpy(im.px.data(), d.data() + i, n);
        } else {
            for (size_t p = 0; p < n; ++p) {
                const uint16_t v = (uint16_t)((d[i + 2 * p] << 8) | d[i + 2 * p + 1]);
                std::memcpy(im.px.data() + 2 * p, &v, 2);
            }
        }
    } else {
        for (size_t p = 0; p < n; ++p) {
            long v;
            if (!pgm_token(d, i, v) || v > maxv) return fail("bad ASCII PGM sample", path);
            if (im.dtype == IWPP_U8) {
                im.px[p] = (unsigned char)v;
            } else {
                const uint16_t s = (uint16_t)v;
                std::memcpy(im.px.data() + 2 * p, &s, 2);
            }
        }
    }
    return true;
}

bool write_pgm(const std::string& path, const Image& im) {
    if (im.dtype == IWPP_I32) return fail("PGM holds 8- or 16-bit pixels only", path);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail("cannot write", path);
    std::fprintf(f, "P5\n%d %d\n%d\n", im.w, im.h, im.dtype == IWPP_U8 ? 255 : 65535);
    bool ok = true;
    if (im.dtype == IWPP_U8) {
        ok = std::fwrite(im.px.data(), 1, im.px.size(), f) == im.px.size();
    } else {
        std::vector<unsigned char> be(im.px.size());
        for (size_t p = 0; p < im.px.size() / 2; ++p) {
            uint16_t v;
            std::memcpy(&v, im.px.data() + 2 * p, 2);
            be[2 * p] = (unsigned char)(v >> 8);
            be[2 * p + 1] = (unsigned char)(v & 0xff);
        }
        ok = std::fwrite(be.data(), 1, be.size(), f) == be.size();
    }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? true : fail("write failed", path);
}

// ---- TIFF: baseline uncompressed grayscale, 8 / 16 / 32 bits per sample
uint32_t rd(const std::vector<unsigned char>& d, size_t off, int bytes, bool le) {
    uint32_t v = 0;
    for (int b = 0; b < bytes; ++b) {
        const uint32_t byte = d[off + (size_t)b];
        v |= le ? byte << (8 * b) : byte << (8 * (bytes - 1 - b));
    }
    return v;
}

bool read_tiff(const std::string& path, const std::vector<unsigned char>& d, Image& im) {
    if (d.size() < 8) return fail("not a TIFF file", path);
    const bool le = d[0] == 'I' && d[1] == 'I';
    if (!le && !(d[0] == 'M' && d[1] == 'M')) return fail("not a TIFF file", path);
    if (rd(d, 2, 2, le) != 42) return fail("not a TIFF file", path);
    const size_t ifd = rd(d, 4, 4, le);
    if (ifd + 2 > d.size()) return fail("bad TIFF directory", path);
    const unsigned nent = rd(d, ifd, 2, le);
    if (ifd + 2 + 12ull * nent > d.size()) return fail("bad TIFF directory", path);
    long w = -1, h = -1, bits = 8, comp = 1, spp = 1, fmt = 1, rows_per_strip = -1;
    std::vector<uint32_t> offs, counts;
    for (unsigned e = 0; e < nent; ++e) {
        const size_t p = ifd + 2 + 12ull * e;
        const unsigned tag = rd(d, p, 2, le), type = rd(d, p + 2, 2, le);
        const uint32_t cnt = rd(d, p + 4, 4, le);
        const int sz = type == 3 ? 2 : type == 4 ? 4 : type == 1 ? 1 : 0;
        if (sz == 0) continue;
        auto value = [&](uint32_t k) -> uint32_t {
            const size_t base = (size_t)sz * cnt <= 4 ? p + 8 : rd(d, p + 8, 4, le);
            if (base + (size_t)sz * (k + 1) > d.size()) return 0;
            return rd(d, base + (size_t)sz * k, sz, le);
        };
        switch (tag) {
            case 256: w = value(0); break;
            case 257: h = value(0); break;
            case 258: bits = value(0); break;
            case 259: comp = value(0); break;
            case 277: spp = value(0); break;
            case 278: rows_per_strip = value(0); break;
            case 339: fmt = value(0); break;
            case 273:
                for (uint32_t k = 0; k < cnt && k < (1u << 24); ++k) offs.push_back(value(k));
                break;
            case 279:
                for (uint32_t k = 0; k < cnt && k < (1u << 24); ++k) counts.push_back(value(k));
                break;
            default: break;
        }
    }
    if (w <= 0 || h <= 0 || comp != 1 || spp != 1 || offs.empty() || offs.size() != counts.size())
        return fail("unsupported TIFF (grayscale, uncompressed only)", path);
    if (bits == 8 && fmt == 1) im.dtype = IWPP_U8;
    else if (bits == 16 && fmt == 1) im.dtype = IWPP_U16;
    else if (bits == 32 && fmt == 2) im.dtype = IWPP_I32;
    else return fail("unsupported TIFF sample format", path);
    (void)rows_per_strip;
    im.w = (int)w;
    im.h = (int)h;
    const size_t total = (size_t)w * h * im.bpp();
    im.px.clear();
    for (size_t s = 0; s < offs.size(); ++s) {
        if ((size_t)offs[s] + counts[s] > d.size()) return fail("TIFF strip out of range", path);
        im.px.insert(im.px.end(), d.begin() + offs[s], d.begin() + offs[s] + counts[s]);
    }
    if (im.px.size() < total) return fail("TIFF data too short", path);
    im.px.resize(total);
    if (!le && im.bpp() > 1) {  // to host (little-endian) order
        for (size_t p = 0; p < total; p += im.bpp()) std::reverse(im.px.begin() + p, im.px.begin() + p + im.bpp());
    }
    return true;
}

bool write_tiff(const std::string& path, const Image& im) {
    // little-endian, one strip, entries sorted by tag
    const uint32_t nbytes = (uint32_t)im.px.size();
    const uint16_t bits = (uint16_t)(8 * im.bpp());
    const uint16_t fmt = im.dtype == IWPP_I32 ? 2 : 1;
    const uint32_t data_off = 8;
    const uint32_t ifd_off = data_off + nbytes + (nbytes & 1u);
    struct Ent { uint16_t tag, type; uint32_t count, value; };
    const Ent ents[] = {{256, 4, 1, (uint32_t)im.w}, {257, 4, 1, (uint32_t)im.h}, {258, 3, 1, bits},
                        {259, 3, 1, 1},   {262, 3, 1, 1},  {273, 4, 1, data_off},
                        {277, 3, 1, 1},   {278, 4, 1, (uint32_t)im.h}, {279, 4, 1, nbytes},
                        {339, 3, 1, fmt}};
    std::vector<unsigned char> out;
    auto put = [&](uint32_t v, int bytes) {
        for (int b = 0; b < bytes; ++b) out.push_back((unsigned char)(v >> (8 * b)));
    };
    out.push_back('I');
    out.push_back('I');
    put(42, 2);
    put(ifd_off, 4);
    out.insert(out.end(), im.px.begin(), im.px.end());
    if (nbytes & 1u) out.push_back(0);
    const uint16_t n = (uint16_t)(sizeof(ents) / sizeof(ents[0]));
    put(n, 2);
    for (const Ent& e : ents) {
        put(e.tag, 2);
        put(e.type, 2);
        put(e.count, 4);
        put(e.value, 4);  // SHORT values sit in the low bytes (little-endian)
    }
    put(0, 4);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail("cannot write", path);
    bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? true : fail("write failed", path);
}

// ---- raw: sizes and type from --raw WxH:type
bool read_raw(const std::string& path, const std::vector<unsigned char>& d, const std::string& spec, Image& im) {
    int w = 0, h = 0;
    char t[8] = {0};
    if (spec.empty() || std::sscanf(spec.c_str(), "%dx%d:%7s", &w, &h, t) != 3 || w <= 0 || h <= 0)
        return fail("raw input needs --raw WxH:u8|u16|i32", path);
    const std::string ts(t);
    im.dtype = ts == "u8" ? IWPP_U8 : ts == "u16" ? IWPP_U16 : ts == "i32" ? IWPP_I32 : -1;
    if (im.dtype < 0) return fail("raw type must be u8, u16 or i32", path);
    im.w = w;
    im.h = h;
    const size_t total = (size_t)w * h * im.bpp();
    if (d.size() < total) return fail("raw file too short", path);
    im.px.assign(d.begin(), d.begin() + total);
    return true;
}

bool load(const std::string& path, const std::string& raw_spec, Image& im) {
    std::vector<unsigned char> d;
    if (!read_file(path, d)) return fail("cannot read", path);
    if (d.size() >= 2 && d[0] == 'P' && (d[1] == '5' || d[1] == '2')) return read_pgm(path, d, im);
    if (d.size() >= 4 && ((d[0] == 'I' && d[1] == 'I') || (d[0] == 'M' && d[1] == 'M'))) return read_tiff(path, d, im);
    return read_raw(path, d, raw_spec, im);
}

bool save(const std::string& path, const Image& im) {
    if (ends_with(path, ".pgm")) return write_pgm(path, im);
    if (ends_with(path, ".tif") || ends_with(path, ".tiff")) return write_tiff(path, im);
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return fail("cannot write", path);
    bool ok = std::fwrite(im.px.data(), 1, im.px.size(), f) == im.px.size();
    ok = (std::fclose(f) == 0) && ok;
    return ok ? true : fail("write failed", path);
}

int usage() {
    std::fprintf(stderr,
                 "usage: iwpp_cli <marker> <mask> <output> <usePGMLoader> [--conn 4|8] [--variant V]\n"
                 "                [--raw WxH:u8|u16|i32] [--no-clip] [--repeat N]\n"
                 "                [--init-passes N] [--solver 0|1|2] [--tile-rows 32|64]\n"
                 "       iwpp_cli --convert <in> <out> [--raw WxH:type]\n");
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    std::vector<std::string> pos;
    int conn = 4, variant = IWPP_QUEUE_DEFAULT, repeat = 1;
    iwpp_config cfg{};
    cfg.init_passes = -1;
    bool clip = true, convert = false;
    std::string raw_spec;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        if (a == "--conn" && i + 1 < argc) {
            conn = std::atoi(argv[++i]);
        } else if (a == "--variant" && i + 1 < argc) {
            const std::string v = argv[++i];
            variant = v == "mutex" ? IWPP_QUEUE_MUTEX : v == "double" ? IWPP_QUEUE_DOUBLE
                    : v == "unique" ? IWPP_QUEUE_UNIQUE : v == "async" ? IWPP_QUEUE_ASYNC : IWPP_QUEUE_DEFAULT;
        } else if (a == "--raw" && i + 1 < argc) {
            raw_spec = argv[++i];
        } else if (a == "--init-passes" && i + 1 < argc) {
            cfg.init_passes = std::atoi(argv[++i]);
        } else if (a == "--solver" && i + 1 < argc) {
            cfg.solver = std::atoi(argv[++i]);
        } else if (a == "--tile-rows" && i + 1 < argc) {
            cfg.tile_rows = std::atoi(argv[++i]);
        } else if (a == "--no-clip") {
            clip = false;
        } else if (a == "--repeat" && i + 1 < argc) {
            repeat = std::max(1, std::atoi(argv[++i]));
        } else if (a == "--convert") {
            convert = true;
        } else {
            pos.push_back(a);
        }
    }
    if (convert) {
        if (pos.size() != 2) return usage();
        Image im;
        if (!load(pos[0], raw_spec, im) || !save(pos[1], im)) return 2;
        return 0;
    }
    if (pos.size() < 4) return usage();
    if (conn != 4 && conn != 8) return usage();
    Image marker, mask;
    if (!load(pos[0], raw_spec, marker) || !load(pos[1], raw_spec, mask)) return 2;
    if (marker.w != mask.w || marker.h != mask.h || marker.dtype != mask.dtype) {
        std::fprintf(stderr, "iwpp_cli: marker and mask differ in size or pixel type\n");
        return 2;
    }
    const size_t row = (size_t)marker.w * marker.bpp();
    void *d_marker = nullptr, *d_mask = nullptr, *d_pristine = nullptr;
    size_t pm = 0, pk = 0, pp = 0;
    cudaError_t e = cudaMallocPitch(&d_marker, &pm, row, (size_t)marker.h);
    if (e == cudaSuccess) e = cudaMallocPitch(&d_mask, &pk, row, (size_t)marker.h);
    if (e == cudaSuccess && repeat > 1) e = cudaMallocPitch(&d_pristine, &pp, row, (size_t)marker.h);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(d_marker, pm, marker.px.data(), row, row, (size_t)marker.h, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(d_mask, pk, mask.px.data(), row, row, (size_t)marker.h, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "iwpp_cli: %s\n", cudaGetErrorString(e));
        return 3;
    }
    int rc = IWPP_OK;
    if (clip) rc = iwpp_clip(d_marker, d_mask, pm, pk, marker.w, marker.h, marker.dtype, nullptr);
    if (rc == IWPP_OK && d_pristine)
        e = cudaMemcpy2D(d_pristine, pp, d_marker, pm, row, (size_t)marker.h, cudaMemcpyDeviceToDevice);
    iwpp_handle h = nullptr;
    if (rc == IWPP_OK) rc = iwpp_handle_create(&h, 0);
    std::vector<double> times;
    for (int r = 0; r < repeat && rc == IWPP_OK; ++r) {
        if (r > 0)
            cudaMemcpy2D(d_marker, pm, d_pristine, pp, row, (size_t)marker.h, cudaMemcpyDeviceToDevice);
        cudaDeviceSynchronize();
        const auto t0 = std::chrono::high_resolution_clock::now();
        rc = iwpp_reconstruct(h, d_marker, d_mask, pm, pk, marker.w, marker.h, marker.dtype, conn, variant, &cfg,
                              nullptr, nullptr);
        const auto t1 = std::chrono::high_resolution_clock::now();
        times.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    if (rc != IWPP_OK) {
        std::fprintf(stderr, "iwpp_cli: %s\n", iwpp_status_string(rc));
        return 4;
    }
    std::sort(times.begin(), times.end());
    const double ms = times[times.size() / 2];
    std::printf("Tempo de execução: %ld\n", (long)ms);
    std::fprintf(stderr, "iwpp_cli: %dx%d %s %d-conn, %.3f ms (median of %d)\n", marker.w, marker.h,
                 marker.dtype == IWPP_U8 ? "uint8" : marker.dtype == IWPP_U16 ? "uint16" : "int32", conn, ms, repeat);
    Image out = marker;
    e = cudaMemcpy2D(out.px.data(), row, d_marker, pm, row, (size_t)marker.h, cudaMemcpyDeviceToHost);
    iwpp_handle_destroy(h);
    cudaFree(d_marker);
    cudaFree(d_mask);
    if (d_pristine) cudaFree(d_pristine);
    if (e != cudaSuccess) return 3;
    return save(pos[2], out) ? 0 : 2;
}
