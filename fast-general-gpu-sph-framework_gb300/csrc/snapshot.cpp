// Snapshot / restart file format (host only).
//
// The reference has no restart path: its scene always starts from the JSON
// lattice (sph_hybrid_system.cpp:432-473). A snapshot stores what a handle
// needs to continue a run bit for bit: every scene's parameter set and
// particle count, and the particle state (position with w = 1/rho, velocity,
// evaluated velocity with w = pressure) in the handle's current order. The
// next frame re-sorts the particles by (micro key, current index), which is
// exactly what the uninterrupted run does, so a restarted handle produces the
// same bits as the original one.
//
// Layout (little-endian, version 1):
//   header (88 bytes, SnapshotHeader)
//   gsph_params[n_scenes]          (params_bytes each)
//   uint32 counts[n_scenes]
//   float4 pos[n], vel[n], ev[n]   (n = sum of counts)
// The header's checksum is a 64-bit FNV-1a over the payload's 8-byte words
// (the payload is padded with zero bytes to a multiple of 8 for hashing).

#include <cstdio>
#include <cstring>
#include <vector>

#include "gsph_internal.h"

namespace gsph {

namespace {

constexpr char kMagic[8] = {'G', 'S', 'P', 'H', 'S', 'N', 'A', 'P'};
constexpr uint32_t kVersion = 1;

struct SnapshotHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    uint32_t params_bytes;
    uint32_t n_scenes;
    uint64_t n_particles;
    uint64_t frames;
    uint64_t payload_bytes;
    uint64_t checksum;
    uint32_t flags;
    uint32_t reserved[7];
};
static_assert(sizeof(SnapshotHeader) == 88, "snapshot header layout");

struct Hasher {
    uint64_t h = 0xcbf29ce484222325ull;
    unsigned char tail[8] = {0};
    int nt = 0;
    void add(const void *data, size_t bytes) {
        const unsigned char *p = static_cast<const unsigned char *>(data);
        while (bytes && nt) {
            tail[nt++] = *p++;
            --bytes;
            if (nt == 8) word(tail);
        }
        while (bytes >= 8) {
            word(p);
            p += 8;
            bytes -= 8;
        }
        while (bytes) {
            tail[nt++] = *p++;
            --bytes;
        }
    }
    void word(const unsigned char *w) {
        uint64_t v;
        std::memcpy(&v, w, 8);
        h = (h ^ v) * 0x100000001b3ull;
        nt = 0;
    }
    uint64_t finish() {
        if (nt) {
            std::memset(tail + nt, 0, size_t(8 - nt));
            word(tail);
        }
        return h;
    }
};

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

}  // namespace

gsph_status snapshot_write(const char *path, const gsph_params *plist,
                           const uint32_t *counts, uint32_t n_scenes,
                           const float *pos4, const float *vel4, const float *ev4,
                           uint64_t frames) {
    if (!path || (n_scenes && (!plist || !counts))) {
        set_error("gsph_snapshot_save: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    uint64_t n = 0;
    for (uint32_t k = 0; k < n_scenes; ++k) n += counts[k];
    if (n && (!pos4 || !vel4 || !ev4)) {
        set_error("gsph_snapshot_save: null state");
        return GSPH_ERR_INVALID_ARG;
    }
    SnapshotHeader hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.version = kVersion;
    hd.header_bytes = sizeof(SnapshotHeader);
    hd.params_bytes = sizeof(gsph_params);
    hd.n_scenes = n_scenes;
    hd.n_particles = n;
    hd.frames = frames;
    const size_t state = size_t(n) * 16;
    hd.payload_bytes = uint64_t(n_scenes) * (sizeof(gsph_params) + 4) + 3 * state;
    Hasher hs;
    hs.add(plist, size_t(n_scenes) * sizeof(gsph_params));
    hs.add(counts, size_t(n_scenes) * 4);
    hs.add(pos4, state);
    hs.add(vel4, state);
    hs.add(ev4, state);
    hd.checksum = hs.finish();
    File fl;
    fl.f = std::fopen(path, "wb");
    if (!fl.f) {
        set_error("gsph_snapshot_save: cannot open %s for writing", path);
        return GSPH_ERR_IO;
    }
    bool ok = std::fwrite(&hd, sizeof hd, 1, fl.f) == 1;
    if (n_scenes) {
        ok = ok && std::fwrite(plist, sizeof(gsph_params), n_scenes, fl.f) == n_scenes;
        ok = ok && std::fwrite(counts, 4, n_scenes, fl.f) == n_scenes;
    }
    if (n) {
        ok = ok && std::fwrite(pos4, 16, size_t(n), fl.f) == size_t(n);
        ok = ok && std::fwrite(vel4, 16, size_t(n), fl.f) == size_t(n);
        ok = ok && std::fwrite(ev4, 16, size_t(n), fl.f) == size_t(n);
    }
    ok = (std::fclose(fl.f) == 0) && ok;
    fl.f = nullptr;
    if (!ok) {
        set_error("gsph_snapshot_save: write to %s failed", path);
        return GSPH_ERR_IO;
    }
    return GSPH_OK;
}

static gsph_status read_header(FILE *f, const char *path, SnapshotHeader &hd) {
    if (std::fread(&hd, sizeof hd, 1, f) != 1) {
        set_error("snapshot %s: truncated header", path);
        return GSPH_ERR_IO;
    }
    if (std::memcmp(hd.magic, kMagic, 8) != 0) {
        set_error("snapshot %s: not a gsph snapshot", path);
        return GSPH_ERR_PARSE;
    }
    if (hd.version != kVersion || hd.header_bytes != sizeof(SnapshotHeader) ||
        hd.params_bytes != sizeof(gsph_params)) {
        set_error("snapshot %s: version %u (header %u B, params %u B) is not "
                  "version %u (%zu B, %zu B)",
                  path, hd.version, hd.header_bytes, hd.params_bytes, kVersion,
                  sizeof(SnapshotHeader), sizeof(gsph_params));
        return GSPH_ERR_PARSE;
    }
    if (hd.n_scenes > 1000000u || hd.n_particles > 0x7FFFFFFFull ||
        hd.payload_bytes != uint64_t(hd.n_scenes) * (sizeof(gsph_params) + 4) +
                                3ull * 16ull * hd.n_particles) {
        set_error("snapshot %s: inconsistent header", path);
        return GSPH_ERR_PARSE;
    }
    return GSPH_OK;
}

gsph_status snapshot_header(const char *path, uint32_t *n_scenes,
                            uint64_t *n_particles, uint64_t *frames) {
    if (!path) {
        set_error("gsph_snapshot_info: null path");
        return GSPH_ERR_INVALID_ARG;
    }
    File fl;
    fl.f = std::fopen(path, "rb");
    if (!fl.f) {
        set_error("snapshot %s: cannot open", path);
        return GSPH_ERR_IO;
    }
    SnapshotHeader hd;
    gsph_status st = read_header(fl.f, path, hd);
    if (st) return st;
    if (n_scenes) *n_scenes = hd.n_scenes;
    if (n_particles) *n_particles = hd.n_particles;
    if (frames) *frames = hd.frames;
    return GSPH_OK;
}

gsph_status snapshot_read(const char *path, std::vector<gsph_params> &plist,
                          std::vector<uint32_t> &counts, std::vector<float> &pos4,
                          std::vector<float> &vel4, std::vector<float> &ev4,
                          uint64_t &frames) {
    if (!path) {
        set_error("gsph_snapshot_load: null path");
        return GSPH_ERR_INVALID_ARG;
    }
    File fl;
    fl.f = std::fopen(path, "rb");
    if (!fl.f) {
        set_error("snapshot %s: cannot open", path);
        return GSPH_ERR_IO;
    }
    SnapshotHeader hd;
    gsph_status st = read_header(fl.f, path, hd);
    if (st) return st;
    const size_t S = hd.n_scenes, n = size_t(hd.n_particles);
    plist.resize(S);
    counts.resize(S);
    pos4.resize(n * 4);
    vel4.resize(n * 4);
    ev4.resize(n * 4);
    bool ok = true;
    if (S) {
        ok = ok && std::fread(plist.data(), sizeof(gsph_params), S, fl.f) == S;
        ok = ok && std::fread(counts.data(), 4, S, fl.f) == S;
    }
    if (n) {
        ok = ok && std::fread(pos4.data(), 16, n, fl.f) == n;
        ok = ok && std::fread(vel4.data(), 16, n, fl.f) == n;
        ok = ok && std::fread(ev4.data(), 16, n, fl.f) == n;
    }
    if (!ok) {
        set_error("snapshot %s: truncated payload", path);
        return GSPH_ERR_IO;
    }
    uint64_t total = 0;
    for (uint32_t c : counts) total += c;
    if (total != hd.n_particles) {
        set_error("snapshot %s: scene counts sum to %llu, header says %llu", path,
                  (unsigned long long)total, (unsigned long long)hd.n_particles);
        return GSPH_ERR_PARSE;
    }
    Hasher hs;
    hs.add(plist.data(), S * sizeof(gsph_params));
    hs.add(counts.data(), S * 4);
    hs.add(pos4.data(), n * 16);
    hs.add(vel4.data(), n * 16);
    hs.add(ev4.data(), n * 16);
    if (hs.finish() != hd.checksum) {
        set_error("snapshot %s: checksum mismatch (file corrupted)", path);
        return GSPH_ERR_PARSE;
    }
    frames = hd.frames;
    return GSPH_OK;
}

}  // namespace gsph
