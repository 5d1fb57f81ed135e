// Partio BGEO particle files: the record packing on the device and the file writer.
//
// The layout is the one partio's BGEO writer produces for the reference's
// ParticleExporter_Partio (Simulator/Exporter/ParticleExporter_Partio.cpp:67-201) and its
// particle state files (Simulator/SimulatorBase.cpp:2062-2192); partio is vendored in the
// reference tree (extern/partio), and the format is restated here in this project's own code.
// All numbers are big-endian:
//   int32 magic "Bgeo", char 'V', int32 version 5, int32 points, primitives 0, point groups 0,
//   primitive groups 0, point attributes, vertex attributes 0, primitive attributes 0,
//   detail attributes 0;
//   per point attribute (all but the position): uint16 name length, name, uint16 size,
//   int32 type (0 FLOAT, 1 INT, 5 VECTOR), size x int32 0 (the defaults);
//   per point: float x, y, z, 1, then each attribute's values (float or int32);
//   the end marker bytes 0x00 0xff.
// With compression the whole file is one gzip member (RFC 1952), as partio writes it when the
// reference asks for compression.  The member is compressed in independent pieces on all host
// cores but one: every piece but the last ends with a sync flush (byte-aligned, not final), so the
// concatenated raw deflate streams form one valid stream, and the pieces' CRC-32 values are
// combined into the member's (zlib crc32_combine).  zlib is loaded at run time.
#include "bgeo.h"

#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>

#include "../../include/sphgb300.h"

#if __has_include(<zlib.h>)
#include <zlib.h>
#define SPHGB_HAVE_ZLIB 1
#else
#define SPHGB_HAVE_ZLIB 0
#endif

namespace sphgb {

namespace {

struct BgeoPackParams {
    const void *src[kBgeoMaxColumns];
    uint32_t comps[kBgeoMaxColumns];
    uint32_t kind[kBgeoMaxColumns];
    uint8_t col[kBgeoMaxWords];    // column group of record word w
    uint8_t comp[kBgeoMaxWords];   // its component
    uint32_t words;
    uint32_t n;
};

__global__ void k_bgeo_pack(BgeoPackParams p, uint32_t *__restrict__ out)
{
    const size_t total = (size_t)p.n * p.words;
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(k / p.words), w = (uint32_t)(k % p.words);
        const uint32_t c = p.col[w];
        const size_t e = (size_t)i * p.comps[c] + p.comp[w];
        uint32_t v;
        switch (p.kind[c]) {
        case 0:
        case 2: v = static_cast<const uint32_t *>(p.src[c])[e]; break;
        case 1: v = __float_as_uint((float)static_cast<const double *>(p.src[c])[e]); break;
        default: v = __float_as_uint(1.0f); break;
        }
        out[k] = __byte_perm(v, 0, 0x0123);
    }
}

}  // namespace

void launch_bgeo_pack(const BgeoColumn *cols, uint32_t ncols, uint32_t n, uint32_t *out, cudaStream_t s)
{
    BgeoPackParams p{};
    uint32_t w = 0;
    for (uint32_t c = 0; c < ncols && c < kBgeoMaxColumns; c++) {
        p.src[c] = cols[c].src;
        p.comps[c] = cols[c].comps;
        p.kind[c] = cols[c].kind;
        for (uint32_t m = 0; m < cols[c].comps && w < kBgeoMaxWords; m++, w++) {
            p.col[w] = (uint8_t)c;
            p.comp[w] = (uint8_t)m;
        }
    }
    p.words = w;
    p.n = n;
    const size_t total = (size_t)n * w;
    if (!total) return;
    const size_t blocks = std::min<size_t>((total + 255) / 256, 152u * 16u);
    k_bgeo_pack<<<(unsigned)blocks, 256, 0, s>>>(p, out);
}

namespace {

void put_be32(std::vector<unsigned char> &b, uint32_t v)
{
    for (int s = 24; s >= 0; s -= 8) b.push_back((unsigned char)(v >> s));
}
void put_be16(std::vector<unsigned char> &b, uint16_t v)
{
    b.push_back((unsigned char)(v >> 8));
    b.push_back((unsigned char)v);
}

std::vector<unsigned char> bgeo_header(uint32_t n, const std::vector<BgeoAttr> &attrs)
{
    std::vector<unsigned char> h;
    put_be32(h, ((uint32_t)'B' << 24) | ((uint32_t)'g' << 16) | ((uint32_t)'e' << 8) | (uint32_t)'o');
    h.push_back((unsigned char)'V');
    put_be32(h, 5u);
    put_be32(h, n);
    put_be32(h, 0u);                        // primitives
    put_be32(h, 0u);                        // point groups
    put_be32(h, 0u);                        // primitive groups
    put_be32(h, (uint32_t)attrs.size());    // point attributes besides the position
    put_be32(h, 0u);                        // vertex attributes
    put_be32(h, 0u);                        // primitive attributes
    put_be32(h, 0u);                        // detail attributes
    for (const BgeoAttr &a : attrs) {
        put_be16(h, (uint16_t)a.name.size());
        h.insert(h.end(), a.name.begin(), a.name.end());
        put_be16(h, (uint16_t)a.comps);
        put_be32(h, a.integer ? 1u : (a.comps == 3 ? 5u : 0u));
        for (uint32_t k = 0; k < a.comps; k++) put_be32(h, 0u);
    }
    return h;
}

const unsigned char kBgeoEnd[2] = {0x00, 0xff};

#if SPHGB_HAVE_ZLIB
struct ZlibApi {
    int (*deflate_init2)(z_streamp, int, int, int, int, int, const char *, int) = nullptr;
    int (*deflate_)(z_streamp, int) = nullptr;
    int (*deflate_end)(z_streamp) = nullptr;
    uLong (*deflate_bound)(z_streamp, uLong) = nullptr;
    uLong (*crc)(uLong, const Bytef *, uInt) = nullptr;
    uLong (*crc_combine)(uLong, uLong, z_off_t) = nullptr;
    int (*inflate_init2)(z_streamp, int, const char *, int) = nullptr;
    int (*inflate_)(z_streamp, int) = nullptr;
    int (*inflate_end)(z_streamp) = nullptr;
    int (*inflate_reset)(z_streamp) = nullptr;
    bool ok = false;
    bool inflate_ok = false;
};

const ZlibApi &zlib_api()
{
    static const ZlibApi api = [] {
        ZlibApi a;
        void *h = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
        if (!h) h = dlopen("libz.so", RTLD_NOW | RTLD_LOCAL);
        if (!h) return a;
        a.deflate_init2 = reinterpret_cast<decltype(a.deflate_init2)>(dlsym(h, "deflateInit2_"));
        a.deflate_ = reinterpret_cast<decltype(a.deflate_)>(dlsym(h, "deflate"));
        a.deflate_end = reinterpret_cast<decltype(a.deflate_end)>(dlsym(h, "deflateEnd"));
        a.deflate_bound = reinterpret_cast<decltype(a.deflate_bound)>(dlsym(h, "deflateBound"));
        a.crc = reinterpret_cast<decltype(a.crc)>(dlsym(h, "crc32"));
        a.crc_combine = reinterpret_cast<decltype(a.crc_combine)>(dlsym(h, "crc32_combine"));
        a.ok = a.deflate_init2 && a.deflate_ && a.deflate_end && a.deflate_bound && a.crc && a.crc_combine;
        a.inflate_init2 = reinterpret_cast<decltype(a.inflate_init2)>(dlsym(h, "inflateInit2_"));
        a.inflate_ = reinterpret_cast<decltype(a.inflate_)>(dlsym(h, "inflate"));
        a.inflate_end = reinterpret_cast<decltype(a.inflate_end)>(dlsym(h, "inflateEnd"));
        a.inflate_reset = reinterpret_cast<decltype(a.inflate_reset)>(dlsym(h, "inflateReset"));
        a.inflate_ok = a.inflate_init2 && a.inflate_ && a.inflate_end && a.inflate_reset;
        return a;
    }();
    return api;
}

struct Piece {
    const unsigned char *in;
    size_t len;
    bool last;
    std::vector<unsigned char> out;
    uLong crc = 0;
    bool ok = false;
};

// one raw deflate stream ending in a sync flush (or, for the last piece, the final block)
void deflate_piece(const ZlibApi &z, Piece &pc, int level)
{
    z_stream s;
    std::memset(&s, 0, sizeof s);
    if (z.deflate_init2(&s, level, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY, ZLIB_VERSION, (int)sizeof(z_stream)) != Z_OK)
        return;
    pc.out.resize(z.deflate_bound(&s, (uLong)pc.len) + 64);
    s.next_in = const_cast<Bytef *>(pc.in);
    s.avail_in = (uInt)pc.len;
    const int flush = pc.last ? Z_FINISH : Z_SYNC_FLUSH;
    size_t done = 0;
    bool ok = false;
    for (int guard = 0; guard < 64; guard++) {
        s.next_out = pc.out.data() + done;
        s.avail_out = (uInt)(pc.out.size() - done);
        const int r = z.deflate_(&s, flush);
        done = pc.out.size() - s.avail_out;
        if (r == Z_STREAM_ERROR) break;
        if (pc.last ? r == Z_STREAM_END : (s.avail_in == 0 && s.avail_out != 0)) {
            ok = true;
            break;
        }
        pc.out.resize(pc.out.size() * 2);
    }
    z.deflate_end(&s);
    pc.out.resize(done);
    pc.crc = z.crc(0ul, pc.in, (uInt)pc.len);
    pc.ok = ok;
}

void put_le32(unsigned char *p, uint32_t v)
{
    for (int k = 0; k < 4; k++) p[k] = (unsigned char)(v >> (8 * k));
}
#endif

constexpr size_t kPieceBytes = 1u << 20;

}  // namespace

bool bgeo_compression_available()
{
#if SPHGB_HAVE_ZLIB
    return zlib_api().ok;
#else
    return false;
#endif
}

int write_bgeo_file(const std::string &path, const void *records, uint32_t n, uint32_t words,
                    const std::vector<BgeoAttr> &attrs, int level, std::string &err)
{
    const std::vector<unsigned char> head = bgeo_header(n, attrs);
    const size_t body = (size_t)n * words * 4u;
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        err = "export: cannot open " + path;
        return SPHGB_ERR_ARGUMENT;
    }
    bool ok = true;
    if (level == 0) {
        ok = fwrite(head.data(), 1, head.size(), f) == head.size() &&
             (body == 0 || fwrite(records, 1, body, f) == body) && fwrite(kBgeoEnd, 1, 2, f) == 2;
    } else {
#if SPHGB_HAVE_ZLIB
        const ZlibApi &z = zlib_api();
        std::vector<Piece> pieces;
        pieces.push_back({head.data(), head.size(), false, {}, 0, false});
        const unsigned char *rec = static_cast<const unsigned char *>(records);
        for (size_t a = 0; a < body; a += kPieceBytes)
            pieces.push_back({rec + a, std::min(kPieceBytes, body - a), false, {}, 0, false});
        pieces.push_back({kBgeoEnd, 2, true, {}, 0, false});
        std::atomic<size_t> next{0};
        auto work = [&] {
            for (size_t k; (k = next.fetch_add(1)) < pieces.size();) deflate_piece(z, pieces[k], level);
        };
        // all host cores but one, which stays with the thread that drives the steps
        const unsigned hw = std::thread::hardware_concurrency();
        const size_t nt = std::min<size_t>(pieces.size(), hw > 2 ? hw - 1 : 1);
        std::vector<std::thread> pool;
        for (size_t t = 1; t < nt; t++) pool.emplace_back(work);
        work();
        for (std::thread &t : pool) t.join();
        uLong crc = 0;
        size_t total = 0;
        for (const Piece &pc : pieces) {
            ok = ok && pc.ok;
            crc = total ? z.crc_combine(crc, pc.crc, (z_off_t)pc.len) : pc.crc;
            total += pc.len;
        }
        if (!ok) {
            fclose(f);
            err = "export: compression failed";
            return SPHGB_ERR_ARGUMENT;
        }
        // gzip member header: deflate, no flags, no time stamp, Unix
        const unsigned char gz[10] = {0x1f, 0x8b, 8, 0, 0, 0, 0, 0, 0, 3};
        ok = fwrite(gz, 1, 10, f) == 10;
        for (const Piece &pc : pieces) ok = ok && (pc.out.empty() || fwrite(pc.out.data(), 1, pc.out.size(), f) == pc.out.size());
        unsigned char tail[8];
        put_le32(tail, (uint32_t)crc);
        put_le32(tail + 4, (uint32_t)total);
        ok = ok && fwrite(tail, 1, 8, f) == 8;
#else
        fclose(f);
        err = "export: compressed BGEO needs zlib, which this build does not have";
        return SPHGB_ERR_STATE;
#endif
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) {
        err = "export: write failed for " + path;
        return SPHGB_ERR_ARGUMENT;
    }
    return SPHGB_OK;
}

namespace {

// the gzip members of a file, inflated one after another (zlib detects each gzip header)
bool gunzip_all(const std::vector<unsigned char> &in, std::vector<unsigned char> &out, std::string &err)
{
#if SPHGB_HAVE_ZLIB
    const ZlibApi &z = zlib_api();
    if (!z.inflate_ok) {
        err = "reading a compressed BGEO needs zlib (libz.so.1), which could not be loaded";
        return false;
    }
    z_stream s;
    std::memset(&s, 0, sizeof s);
    if (z.inflate_init2(&s, 15 + 16, ZLIB_VERSION, (int)sizeof(z_stream)) != Z_OK) {
        err = "inflateInit2 failed";
        return false;
    }
    s.next_in = const_cast<Bytef *>(in.data());
    s.avail_in = (uInt)in.size();
    std::vector<unsigned char> buf(1u << 20);
    bool ok = true;
    while (true) {
        s.next_out = buf.data();
        s.avail_out = (uInt)buf.size();
        const int r = z.inflate_(&s, Z_NO_FLUSH);
        out.insert(out.end(), buf.data(), buf.data() + (buf.size() - s.avail_out));
        if (r == Z_STREAM_END) {
            if (s.avail_in == 0) break;
            z.inflate_reset(&s);   // another member follows
            continue;
        }
        if (r != Z_OK && r != Z_BUF_ERROR) { ok = false; break; }
        if (r == Z_BUF_ERROR && s.avail_in == 0) { ok = false; break; }
    }
    z.inflate_end(&s);
    if (!ok) err = "corrupt gzip data";
    return ok;
#else
    (void)in;
    (void)out;
    err = "reading a compressed BGEO needs zlib, which this build does not have";
    return false;
#endif
}

struct BeReader {
    const unsigned char *p, *end;
    bool ok = true;
    uint32_t u32()
    {
        if (end - p < 4) { ok = false; return 0; }
        const uint32_t v = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
        p += 4;
        return v;
    }
    uint16_t u16()
    {
        if (end - p < 2) { ok = false; return 0; }
        const uint16_t v = (uint16_t)((p[0] << 8) | p[1]);
        p += 2;
        return v;
    }
    uint8_t u8()
    {
        if (end - p < 1) { ok = false; return 0; }
        return *p++;
    }
    std::string str()
    {
        const uint16_t len = u16();
        if (!ok || end - p < len) { ok = false; return {}; }
        std::string s(reinterpret_cast<const char *>(p), len);
        p += len;
        return s;
    }
};

}  // namespace

int read_bgeo_file(const std::string &path, BgeoPoints &out, std::string &err)
{
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open " + path;
        return SPHGB_ERR_ARGUMENT;
    }
    std::vector<unsigned char> raw;
    unsigned char chunk[1 << 16];
    for (size_t got; (got = fread(chunk, 1, sizeof chunk, f)) > 0;) raw.insert(raw.end(), chunk, chunk + got);
    fclose(f);
    std::vector<unsigned char> plain;
    if (raw.size() >= 2 && raw[0] == 0x1f && raw[1] == 0x8b) {
        if (!gunzip_all(raw, plain, err)) return SPHGB_ERR_ARGUMENT;
    } else {
        plain.swap(raw);
    }
    BeReader r{plain.data(), plain.data() + plain.size()};
    const uint32_t magic = r.u32();
    const uint8_t vchar = r.u8();
    const uint32_t version = r.u32();
    if (!r.ok || magic != 0x4267656fu || vchar != 'V' || version != 5u) {
        err = path + " is not a version-5 BGEO file";
        return SPHGB_ERR_ARGUMENT;
    }
    const uint32_t npoints = r.u32(), nprims = r.u32(), npgroups = r.u32(), nprgroups = r.u32();
    const uint32_t npattr = r.u32(), nvattr = r.u32(), nprattr = r.u32(), ndetail = r.u32();
    (void)npgroups;
    (void)nprgroups;
    (void)nvattr;
    (void)nprattr;
    (void)ndetail;
    if (!r.ok || nprims != 0) {
        err = path + ": not a particle file (primitives present)";
        return SPHGB_ERR_ARGUMENT;
    }
    out = BgeoPoints{};
    out.n = npoints;
    uint32_t words = 4;   // x, y, z, w
    for (uint32_t a = 0; a < npattr; a++) {
        BgeoAttr at;
        at.name = r.str();
        at.comps = r.u16();
        const uint32_t type = r.u32();
        if (!r.ok || (type != 0 && type != 1 && type != 5)) {
            err = path + ": unsupported point attribute type (only float, int and vector)";
            return SPHGB_ERR_ARGUMENT;
        }
        at.integer = type == 1;
        for (uint32_t k = 0; k < at.comps; k++) r.u32();   // defaults
        out.attrs.push_back(at);
        words += at.comps;
    }
    if (!r.ok || (size_t)(r.end - r.p) < (size_t)npoints * words * 4u) {
        err = path + ": truncated point data";
        return SPHGB_ERR_ARGUMENT;
    }
    out.position.resize((size_t)npoints * 3);
    out.values.assign(out.attrs.size(), {});
    for (size_t a = 0; a < out.attrs.size(); a++) out.values[a].resize((size_t)npoints * out.attrs[a].comps);
    for (uint32_t i = 0; i < npoints; i++) {
        for (int d = 0; d < 3; d++) {
            const uint32_t w = r.u32();
            float x;
            std::memcpy(&x, &w, 4);
            out.position[(size_t)i * 3 + d] = x;
        }
        r.u32();   // homogeneous coordinate
        for (size_t a = 0; a < out.attrs.size(); a++)
            for (uint32_t k = 0; k < out.attrs[a].comps; k++) out.values[a][(size_t)i * out.attrs[a].comps + k] = r.u32();
    }
    return SPHGB_OK;
}

}  // namespace sphgb
