// Solver snapshot file: the state a run needs to continue bit for bit
// (velocity, wall velocities, pressure potential and its warm-start copies,
// markers and their springs, sub-step phase; mid-step also the velocity at
// the start of the step and, in the mixed form, its off-diagonal Helmholtz
// term) in one binary file. The reference has no such format (it prints
// vectors with operator<<, src/dt/vector.h:153-165).
//
// Layout (little endian, as the hosts that run this library are):
//   header   : char magic[8] = "AFMIBSNP", uint32 version = 1, uint32 nsections,
//              int32 nx, ny, nz, n, bc, precision, half, reserved,
//              int64 substeps, double mg_rho
//   sections : nsections times { char name[16] (NUL padded), uint32 dtype
//              (1: float64, 2: int32), uint32 reserved, uint64 count }
//              followed by count elements
// Host-only code: the library writes it from host copies of the device state
// and the tests read it back without a GPU.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace afmib {
namespace snap {

constexpr char kMagic[8] = {'A', 'F', 'M', 'I', 'B', 'S', 'N', 'P'};
constexpr uint32_t kVersion = 1;
enum : uint32_t { kF64 = 1, kI32 = 2 };

struct Header {
    char magic[8];
    uint32_t version, nsections;
    int32_t nx, ny, nz, n, bc, precision, half, reserved;
    int64_t substeps;
    double mg_rho;
};
static_assert(sizeof(Header) == 64, "snapshot header layout");

struct SectionHead {
    char name[16];
    uint32_t dtype, reserved;
    uint64_t count;
};
static_assert(sizeof(SectionHead) == 32, "snapshot section layout");

struct Section {
    uint32_t dtype = 0;
    std::vector<unsigned char> bytes;
    uint64_t count() const { return bytes.size() / (dtype == kF64 ? 8 : 4); }
    const double* f64() const { return reinterpret_cast<const double*>(bytes.data()); }
    const int32_t* i32() const { return reinterpret_cast<const int32_t*>(bytes.data()); }
};

struct Writer {
    Header h{};
    std::vector<std::pair<SectionHead, const void*>> secs;
    void add(const char* name, uint32_t dtype, const void* data, uint64_t count) {
        SectionHead sh{};
        std::strncpy(sh.name, name, sizeof(sh.name) - 1);
        sh.dtype = dtype;
        sh.count = count;
        secs.emplace_back(sh, data);
    }
    // false on an I/O error
    bool write(const char* path) {
        std::memcpy(h.magic, kMagic, 8);
        h.version = kVersion;
        h.nsections = (uint32_t)secs.size();
        FILE* f = std::fopen(path, "wb");
        if (!f) return false;
        bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
        for (auto& s : secs) {
            ok = ok && std::fwrite(&s.first, sizeof(SectionHead), 1, f) == 1;
            const size_t esz = s.first.dtype == kF64 ? 8 : 4;
            if (ok && s.first.count) ok = std::fwrite(s.second, esz, s.first.count, f) == s.first.count;
        }
        ok = (std::fclose(f) == 0) && ok;
        return ok;
    }
};

// Reads a whole snapshot; returns an empty string or the reason it failed.
inline std::string read(const char* path, Header* h, std::map<std::string, Section>* out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return "cannot open the snapshot file";
    std::string err;
    if (std::fread(h, sizeof(*h), 1, f) != 1 || std::memcmp(h->magic, kMagic, 8) != 0) err = "not a snapshot file";
    else if (h->version != kVersion) err = "unsupported snapshot version";
    for (uint32_t k = 0; err.empty() && k < h->nsections; ++k) {
        SectionHead sh;
        if (std::fread(&sh, sizeof(sh), 1, f) != 1) { err = "truncated snapshot"; break; }
        if (sh.dtype != kF64 && sh.dtype != kI32) { err = "bad section type"; break; }
        if (sh.count > (uint64_t(1) << 40)) { err = "bad section size"; break; }
        sh.name[sizeof(sh.name) - 1] = 0;
        Section s;
        s.dtype = sh.dtype;
        s.bytes.resize(sh.count * (sh.dtype == kF64 ? 8 : 4));
        if (sh.count && std::fread(s.bytes.data(), 1, s.bytes.size(), f) != s.bytes.size()) {
            err = "truncated snapshot";
            break;
        }
        (*out)[sh.name] = std::move(s);
    }
    std::fclose(f);
    return err;
}

}  // namespace snap
}  // namespace afmib
