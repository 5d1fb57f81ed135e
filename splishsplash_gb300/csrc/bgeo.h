// Partio BGEO particle files (the reference's ParticleExporter_Partio,
// Simulator/Exporter/ParticleExporter_Partio.cpp:67-201, written there through the partio
// library with compression on): the device packs the per-point records, a host thread writes
// the header and, compressed or not, the file.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace sphgb {

// one column group of the point records, read from a field scattered in particle-id order
struct BgeoColumn {
    const void *src;    // n x comps words (kind 0 / 2: 32-bit, 1: 64-bit); unused for kind 3
    uint32_t comps;
    uint32_t kind;      // 0 float, 1 double (stored as float), 2 uint32 (stored as int), 3 the constant 1.0f
};
constexpr uint32_t kBgeoMaxColumns = 16, kBgeoMaxWords = 64;

// records of n points, words = sum of comps, big-endian 32-bit words: out[i * words + w]
void launch_bgeo_pack(const BgeoColumn *cols, uint32_t ncols, uint32_t n, uint32_t *out, cudaStream_t s);

// a point attribute of the file besides the position: partio FLOAT (1 comp), INT (1) or VECTOR (3)
struct BgeoAttr {
    std::string name;
    uint32_t comps;
    bool integer;
};

// Writes header, the n packed records and the end marker.  level 0: plain; 1-9: one gzip member,
// compressed in parallel pieces.  Returns an SPHGB status; err gets the message.
int write_bgeo_file(const std::string &path, const void *records, uint32_t n, uint32_t words,
                    const std::vector<BgeoAttr> &attrs, int level, std::string &err);

// whether zlib could be loaded (levels 1-9 need it)
bool bgeo_compression_available();

// the points of a BGEO particle file: positions and every point attribute (host-order words)
struct BgeoPoints {
    uint32_t n = 0;
    std::vector<float> position;                 // n x 3
    std::vector<BgeoAttr> attrs;                 // besides the position, in file order
    std::vector<std::vector<uint32_t>> values;   // per attribute: n x comps words (float or int bits)
};

// Reads a version-5 BGEO particle file, plain or gzip-compressed (any number of members), as
// partio's reader does for point attributes of type float, int and vector.  Detail attributes
// after the points are not read.  Returns an SPHGB status; err gets the message.
int read_bgeo_file(const std::string &path, BgeoPoints &out, std::string &err);

}  // namespace sphgb
