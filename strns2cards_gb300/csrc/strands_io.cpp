// Strand file ingest and arclength resampling on the host.
//
// Formats (the reference's hair_loader.cpp:15-218 reads the same three):
//   .bin   int32 strand count; per strand an int32 point count and, per point, 7 float32
//          (x, y, z, nx, ny, nz, label); a strand with two consecutive points closer than
//          1e-4 is dropped.
//   .data  (USC) int32 strand count; per strand an int32 point count and that many xyz;
//          one-point strands are skipped.
//   .hair  "HAIR" header: strand count, point count, flags (bit 1: per-strand segment counts
//          present, bit 2: points present), else a default segment count; header of 128
//          words; per-strand uint16 segment counts; xyz float32 points (segments + 1 per
//          strand).  Without the "HAIR" magic: the ZJU layout (strand count, point count,
//          uint16 point counts, xyz points).
// Strands with fewer than two points are not returned (serialize_strands, :220-259).
// A file that cannot be opened gives no strands (the reference prints and continues);
// a truncated file or counts that overrun the points are errors here (the reference reads
// past them).
//
// Resampling (the reference's :261-307): cumulative FP32 lengths sqrt((dx*dx + dy*dy) + dz*dz)
// normalised by the total, target j at t = j / (T - 1) interpolated between the first
// point whose normalised length exceeds t and the one before; the last point is copied.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "s2c.h"

namespace s2c {
void set_error(const char* fmt, ...);
}

namespace {

struct StrandSet {
    std::vector<int32_t> counts;
    std::vector<float> xyz;
};

struct Reader {
    std::vector<unsigned char> buf;
    size_t pos = 0;
    bool ok = true;
    template <class T> T get() {
        T v{};
        if (pos + sizeof(T) > buf.size()) {
            ok = false;
            pos = buf.size();
            return v;
        }
        std::memcpy(&v, buf.data() + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    bool skip(size_t n) {
        if (pos + n > buf.size()) {
            ok = false;
            pos = buf.size();
            return false;
        }
        pos += n;
        return true;
    }
    bool seek(size_t p) {
        if (p > buf.size()) {
            ok = false;
            return false;
        }
        pos = p;
        return true;
    }
};

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

void push(StrandSet& out, const float* p, int n) {
    if (n < 2) return;
    out.counts.push_back(n);
    out.xyz.insert(out.xyz.end(), p, p + 3 * (size_t)n);
}

s2c_status parse_bin(Reader& r, StrandSet& out) {
    const int32_t ns = r.get<int32_t>();
    std::vector<float> pts;
    for (int32_t i = 0; i < ns && r.ok; ++i) {
        const int32_t np = r.get<int32_t>();
        if (!r.ok) break;
        if (np < 0) {
            s2c::set_error("load_strands: negative point count in .bin strand %d", i);
            return S2C_ERR_INVALID;
        }
        pts.resize(3 * (size_t)np);
        for (int32_t j = 0; j < np; ++j) {
            float v[7];
            for (float& x : v) x = r.get<float>();
            pts[3 * (size_t)j] = v[0];
            pts[3 * (size_t)j + 1] = v[1];
            pts[3 * (size_t)j + 2] = v[2];
        }
        if (!r.ok) break;
        bool valid = true;
        for (int32_t j = 0; j + 1 < np; ++j) {
            const float dx = pts[3 * (size_t)j] - pts[3 * (size_t)j + 3];
            const float dy = pts[3 * (size_t)j + 1] - pts[3 * (size_t)j + 4];
            const float dz = pts[3 * (size_t)j + 2] - pts[3 * (size_t)j + 5];
            if (std::sqrt(dx * dx + dy * dy + dz * dz) < 1e-4f) {
                valid = false;
                break;
            }
        }
        if (valid) push(out, pts.data(), np);
    }
    if (!r.ok) {
        s2c::set_error("load_strands: truncated .bin file");
        return S2C_ERR_INVALID;
    }
    return S2C_OK;
}

s2c_status parse_usc(Reader& r, StrandSet& out) {
    const int32_t ns = r.get<int32_t>();
    std::vector<float> pts;
    for (int32_t i = 0; i < ns && r.ok; ++i) {
        const int32_t np = r.get<int32_t>();
        if (!r.ok) break;
        if (np < 0) {
            s2c::set_error("load_strands: negative point count in .data strand %d", i);
            return S2C_ERR_INVALID;
        }
        pts.resize(3 * (size_t)np);
        for (size_t k = 0; k < pts.size(); ++k) pts[k] = r.get<float>();
        if (np != 1) push(out, pts.data(), np);
    }
    if (!r.ok) {
        s2c::set_error("load_strands: truncated .data file");
        return S2C_ERR_INVALID;
    }
    return S2C_OK;
}

s2c_status parse_hair(Reader& r, StrandSet& out) {
    const bool magic = r.buf.size() >= 4 && std::memcmp(r.buf.data(), "HAIR", 4) == 0;
    uint32_t ns = 0, np_total = 0;
    std::vector<uint16_t> seg;
    bool plus_one = true;
    if (magic) {
        r.skip(4);
        ns = r.get<uint32_t>();
        np_total = r.get<uint32_t>();
        const uint32_t flags = r.get<uint32_t>();
        uint32_t default_seg = 0;
        if (!(flags & 2u)) {
            s2c::set_error("load_strands: .hair file without a points section");
            return S2C_OK;   // the reference reports and returns no strands
        }
        const bool read_default = !(flags & 1u);
        if (read_default) default_seg = r.get<uint32_t>();
        // the reference skips 128 - 3 (or - 4) words past what it has read
        r.skip(4 * (size_t)(128 - (default_seg ? 3 : 4)));
        seg.resize(ns);
        if (default_seg == 0) {
            for (uint32_t i = 0; i < ns; ++i) seg[i] = r.get<uint16_t>();
        } else {
            for (uint32_t i = 0; i < ns; ++i) seg[i] = (uint16_t)default_seg;
        }
    } else {
        plus_one = false;
        ns = r.get<uint32_t>();
        np_total = r.get<uint32_t>();
        seg.resize(ns);
        for (uint32_t i = 0; i < ns; ++i) seg[i] = r.get<uint16_t>();
    }
    if (!r.ok) {
        s2c::set_error("load_strands: truncated .hair header");
        return S2C_ERR_INVALID;
    }
    std::vector<float> pts(3 * (size_t)np_total);
    for (size_t k = 0; k < pts.size(); ++k) pts[k] = r.get<float>();
    if (!r.ok) {
        s2c::set_error("load_strands: truncated .hair points");
        return S2C_ERR_INVALID;
    }
    size_t at = 0;
    for (uint32_t i = 0; i < ns; ++i) {
        const size_t n = (size_t)seg[i] + (plus_one ? 1 : 0);
        if (at + n > np_total) {
            s2c::set_error("load_strands: .hair segment counts overrun the %u points", np_total);
            return S2C_ERR_INVALID;
        }
        push(out, pts.data() + 3 * at, (int)n);
        at += n;
    }
    return S2C_OK;
}

}  // namespace

extern "C" S2C_API s2c_status s2c_load_strands(const char* path, void** handle, int64_t* num_strands,
                                               int64_t* num_points) {
    if (!path || !handle || !num_strands || !num_points) {
        s2c::set_error("load_strands: null argument");
        return S2C_ERR_INVALID;
    }
    *handle = nullptr;
    const std::string p(path);
    const bool bin = ends_with(p, ".bin"), usc = ends_with(p, ".data"), hair = ends_with(p, ".hair");
    if (!bin && !usc && !hair) {
        s2c::set_error("load_strands: unknown file extension.");
        return S2C_ERR_INVALID;
    }
    StrandSet* out = new StrandSet();
    Reader r;
    if (FILE* f = std::fopen(path, "rb")) {
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        r.buf.resize(n > 0 ? (size_t)n : 0);
        if (!r.buf.empty() && std::fread(r.buf.data(), 1, r.buf.size(), f) != r.buf.size()) r.buf.clear();
        std::fclose(f);
        const s2c_status st = bin ? parse_bin(r, *out) : usc ? parse_usc(r, *out) : parse_hair(r, *out);
        if (st != S2C_OK) {
            delete out;
            return st;
        }
    } else {
        s2c::set_error("load_strands: couldn't open %s", path);   // no strands, as the reference
    }
    *num_strands = (int64_t)out->counts.size();
    *num_points = (int64_t)(out->xyz.size() / 3);
    *handle = out;
    return S2C_OK;
}

extern "C" S2C_API s2c_status s2c_strands_take(void* handle, int32_t* num_samples, float* points) {
    StrandSet* s = (StrandSet*)handle;
    if (!s) {
        s2c::set_error("strands_take: null handle");
        return S2C_ERR_INVALID;
    }
    if (num_samples && !s->counts.empty()) std::memcpy(num_samples, s->counts.data(), 4 * s->counts.size());
    if (points && !s->xyz.empty()) std::memcpy(points, s->xyz.data(), 4 * s->xyz.size());
    delete s;
    return S2C_OK;
}

extern "C" S2C_API s2c_status s2c_resample_strands_by_arclength_host(int num_strands, const int32_t* num_samples,
                                                                     const float* points, int target, float* out) {
    if (num_strands < 0 || target < 2 || (num_strands > 0 && (!num_samples || !points || !out))) {
        s2c::set_error("resample_strands_by_arclength: invalid arguments (strands %d, target %d)", num_strands,
                       target);
        return S2C_ERR_INVALID;
    }
    size_t at = 0;
    std::vector<float> len;
    for (int i = 0; i < num_strands; ++i) {
        const int N = num_samples[i];
        if (N < 2) {
            s2c::set_error("resample_strands_by_arclength: strand %d has %d points (need 2)", i, N);
            return S2C_ERR_INVALID;
        }
        const float* p = points + 3 * at;
        len.assign((size_t)N, 0.f);
        for (int j = 1; j < N; ++j) {
            const float dx = p[3 * j] - p[3 * j - 3], dy = p[3 * j + 1] - p[3 * j - 2], dz = p[3 * j + 2] - p[3 * j - 1];
            len[j] = len[j - 1] + std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        const float total = len.back();
        for (float& l : len) l /= total;
        float* o = out + (size_t)i * target * 3;
        for (int j = 0; j + 1 < target; ++j) {
            const float t = (float)j / (float)(target - 1);
            int k = (int)(std::upper_bound(len.begin(), len.end(), t) - len.begin());
            k = std::min(std::max(k, 1), N - 1);
            const float t0 = (len[k] - t) / (len[k] - len[k - 1]);
            const float t1 = (t - len[k - 1]) / (len[k] - len[k - 1]);
            for (int c = 0; c < 3; ++c) o[3 * j + c] = t0 * p[3 * (k - 1) + c] + t1 * p[3 * k + c];
        }
        for (int c = 0; c < 3; ++c) o[3 * (target - 1) + c] = p[3 * (N - 1) + c];
        at += (size_t)N;
    }
    return S2C_OK;
}
