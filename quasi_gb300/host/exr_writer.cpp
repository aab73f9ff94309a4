// exr_writer.cpp - single-part scanline OpenEXR files without compression.
//
// Layout (all integers little-endian):
//   magic 20000630, version 2 (single-part scanline, no flags)
//   header: attributes (name\0 type\0 int32 size, value) ... \0
//     channels (chlist, sorted by name), compression = NONE, dataWindow, displayWindow,
//     lineOrder = INCREASING_Y, pixelAspectRatio = 1, screenWindowCenter = (0, 0),
//     screenWindowWidth = 1
//   line offset table: one uint64 file offset per scanline
//   scanlines: int32 y, int32 byte count, then each channel's samples of the line in
//   channel-list order
#include "exr_writer.hpp"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <string>
#include <vector>

namespace quasi::io {

uint16_t float_to_half(float f) noexcept {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint16_t sign = static_cast<uint16_t>((x >> 16) & 0x8000u);
    const uint32_t a = x & 0x7fffffffu;
    if (a >= 0x7f800000u)  // inf, nan (keep a quiet nan payload bit)
        return static_cast<uint16_t>(sign | 0x7c00u | (a > 0x7f800000u ? 0x200u | ((a >> 13) & 0x3ffu) : 0u));
    if (a >= 0x477ff000u) return static_cast<uint16_t>(sign | 0x7c00u);  // >= 65520 rounds to inf
    const uint32_t e = a >> 23;
    if (e < 113) {  // |f| < 2^-14: half subnormal, value = round(|f| / 2^-24)
        const uint32_t m = (a & 0x7fffffu) | 0x800000u;
        const uint32_t shift = 126u - e;
        if (shift >= 25) return sign;
        uint32_t r = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
        if (rem > halfway || (rem == halfway && (r & 1u))) ++r;
        return static_cast<uint16_t>(sign | r);
    }
    uint32_t r = ((e - 112u) << 10) | ((a & 0x7fffffu) >> 13);
    const uint32_t rem = a & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) ++r;
    return static_cast<uint16_t>(sign | r);
}

namespace {

enum pixel_type : int32_t { k_half = 1, k_float = 2 };

struct channel {
    std::string name;
    pixel_type type;
    const float* data;  // interleaved source
    uint32_t stride;    // floats per pixel in `data`
    uint32_t offset;    // component within a pixel
};

struct bytes {
    std::vector<uint8_t> b;
    void u8(uint8_t v) { b.push_back(v); }
    void u32(uint32_t v) {
        for (int i = 0; i < 4; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
    }
    void i32(int32_t v) { u32(static_cast<uint32_t>(v)); }
    void u64(uint64_t v) {
        for (int i = 0; i < 8; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
    }
    void f32(float v) {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        u32(u);
    }
    void str(const std::string& s) {
        b.insert(b.end(), s.begin(), s.end());
        b.push_back(0);
    }
    void attr(const std::string& name, const std::string& type, const bytes& value) {
        str(name);
        str(type);
        i32(static_cast<int32_t>(value.b.size()));
        b.insert(b.end(), value.b.begin(), value.b.end());
    }
};

std::expected<void, exr_error> prepare_dir(const std::filesystem::path& path) {
    const auto parent = path.parent_path();
    if (!parent.empty()) {
        std::error_code ec;
        std::filesystem::create_directories(parent, ec);
        if (ec) return std::unexpected{exr_error::directory_error};
    }
    return {};
}

std::expected<void, exr_error> write_channels(const std::filesystem::path& path, uint32_t w, uint32_t h,
                                              std::vector<channel> ch) {
    if (auto d = prepare_dir(path); !d) return d;
    std::sort(ch.begin(), ch.end(), [](const channel& a, const channel& b) { return a.name < b.name; });
    bytes f;
    f.u32(20000630u);
    f.u32(2u);
    bytes chlist;
    for (const channel& c : ch) {
        chlist.str(c.name);
        chlist.i32(c.type);
        chlist.u8(0);  // pLinear
        chlist.u8(0);
        chlist.u8(0);
        chlist.u8(0);  // reserved
        chlist.i32(1);  // x sampling
        chlist.i32(1);  // y sampling
    }
    chlist.u8(0);
    f.attr("channels", "chlist", chlist);
    bytes comp;
    comp.u8(0);  // NO_COMPRESSION
    f.attr("compression", "compression", comp);
    bytes win;
    win.i32(0);
    win.i32(0);
    win.i32(static_cast<int32_t>(w) - 1);
    win.i32(static_cast<int32_t>(h) - 1);
    f.attr("dataWindow", "box2i", win);
    f.attr("displayWindow", "box2i", win);
    bytes order;
    order.u8(0);  // INCREASING_Y
    f.attr("lineOrder", "lineOrder", order);
    bytes one;
    one.f32(1.0f);
    f.attr("pixelAspectRatio", "float", one);
    bytes center;
    center.f32(0.0f);
    center.f32(0.0f);
    f.attr("screenWindowCenter", "v2f", center);
    f.attr("screenWindowWidth", "float", one);
    f.u8(0);  // end of header
    const size_t table = f.b.size();
    for (uint32_t y = 0; y < h; ++y) f.u64(0);
    uint32_t line_bytes = 0;
    for (const channel& c : ch) line_bytes += w * (c.type == k_half ? 2u : 4u);
    for (uint32_t y = 0; y < h; ++y) {
        const uint64_t at = f.b.size();
        for (int i = 0; i < 8; ++i) f.b[table + 8 * y + i] = static_cast<uint8_t>(at >> (8 * i));
        f.i32(static_cast<int32_t>(y));
        f.i32(static_cast<int32_t>(line_bytes));
        for (const channel& c : ch) {
            for (uint32_t x = 0; x < w; ++x) {
                const float v = c.data[(static_cast<size_t>(y) * w + x) * c.stride + c.offset];
                if (c.type == k_half) {
                    const uint16_t hv = float_to_half(v);
                    f.u8(static_cast<uint8_t>(hv));
                    f.u8(static_cast<uint8_t>(hv >> 8));
                } else {
                    f.f32(v);
                }
            }
        }
    }
    std::ofstream out(path, std::ios::binary | std::ios::trunc);
    if (!out) return std::unexpected{exr_error::write_failed};
    out.write(reinterpret_cast<const char*>(f.b.data()), static_cast<std::streamsize>(f.b.size()));
    if (!out) return std::unexpected{exr_error::write_failed};
    return {};
}

}  // namespace

std::expected<void, exr_error> write_exr(const std::filesystem::path& path, const Q_readback_result& r) {
    if (!r.data || r.width == 0 || r.height == 0 || r.channels < 4) return std::unexpected{exr_error::invalid_data};
    std::vector<channel> ch;
    const char* names[4] = {"R", "G", "B", "A"};
    for (uint32_t k = 0; k < 4; ++k) ch.push_back({names[k], k_half, r.data, r.channels, k});
    return write_channels(path, r.width, r.height, std::move(ch));
}

std::expected<void, exr_error> write_exr(const std::filesystem::path& path, const Q_readback_aov_result& r) {
    const Q_aov_buffer& beauty = r.buffers[Q_AOV_BEAUTY];
    if (!beauty.data || beauty.width == 0 || beauty.height == 0 || beauty.channels < 4)
        return std::unexpected{exr_error::invalid_data};
    const uint32_t w = beauty.width, h = beauty.height;
    std::vector<channel> ch;
    const char* rgba[4] = {"R", "G", "B", "A"};
    for (uint32_t k = 0; k < 4; ++k) ch.push_back({rgba[k], k_half, beauty.data, beauty.channels, k});
    auto same = [&](const Q_aov_buffer& b) {
        return b.data && b.width == w && b.height == h && b.channels >= 3;
    };
    const Q_aov_buffer& alb = r.buffers[Q_AOV_ALBEDO];
    if (alb.data && !same(alb)) return std::unexpected{exr_error::invalid_data};
    if (alb.data) {
        const char* n[3] = {"albedo.R", "albedo.G", "albedo.B"};
        for (uint32_t k = 0; k < 3; ++k) ch.push_back({n[k], k_half, alb.data, alb.channels, k});
    }
    const Q_aov_buffer& nrm = r.buffers[Q_AOV_NORMAL];
    if (nrm.data && !same(nrm)) return std::unexpected{exr_error::invalid_data};
    if (nrm.data) {
        const char* n[3] = {"normal.X", "normal.Y", "normal.Z"};
        for (uint32_t k = 0; k < 3; ++k) ch.push_back({n[k], k_half, nrm.data, nrm.channels, k});
    }
    const Q_aov_buffer& dep = r.buffers[Q_AOV_DEPTH];
    if (dep.data && !(dep.width == w && dep.height == h && dep.channels >= 1))
        return std::unexpected{exr_error::invalid_data};
    if (dep.data) ch.push_back({"depth.Z", k_float, dep.data, dep.channels, 0});
    return write_channels(path, w, h, std::move(ch));
}

std::filesystem::path make_timestamped_path(const std::filesystem::path& directory) {
    const std::time_t t = std::chrono::system_clock::to_time_t(std::chrono::system_clock::now());
    std::tm local{};
    localtime_r(&t, &local);
    char name[64];
    std::snprintf(name, sizeof(name), "quasi_%04d%02d%02d_%02d%02d%02d.exr", local.tm_year + 1900, local.tm_mon + 1,
                  local.tm_mday, local.tm_hour, local.tm_min, local.tm_sec);
    return directory / name;
}

}  // namespace quasi::io
