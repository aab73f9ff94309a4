// exr_writer.hpp - OpenEXR output for readback images, written from the public OpenEXR
// file layout (single-part scanline image, no compression); no OpenEXR library needed.
//
// Same calls and error codes as the reference host's writer (src/quasi/io/exr_writer.hpp:
// write_exr for a Q_readback_result and for a Q_readback_aov_result, make_timestamped_path):
//   beauty            R, G, B, A           half
//   AOV file          R, G, B, A           half   (beauty)
//                     albedo.R/G/B         half
//                     normal.X/Y/Z         half
//                     depth.Z              float  (from the depth buffer's first channel)
#pragma once

#include "quasi_cuda.h"

#include <cstdint>
#include <expected>
#include <filesystem>

namespace quasi::io {

enum class exr_error {
    invalid_data,     // null data or zero dimensions
    write_failed,     // the file could not be written
    directory_error,  // the output directory could not be created
};

constexpr const char* to_string(exr_error e) noexcept {
    switch (e) {
        case exr_error::invalid_data: return "Invalid readback data";
        case exr_error::write_failed: return "EXR write failed";
        case exr_error::directory_error: return "Could not create output directory";
    }
    return "Unknown error";
}

std::expected<void, exr_error> write_exr(const std::filesystem::path& path, const Q_readback_result& result);
std::expected<void, exr_error> write_exr(const std::filesystem::path& path, const Q_readback_aov_result& result);

// "quasi_YYYYMMDD_HHMMSS.exr" in `directory` (local time).
std::filesystem::path make_timestamped_path(const std::filesystem::path& directory = ".");

// IEEE binary16 from binary32, round to nearest even (NaN stays NaN, overflow -> inf).
uint16_t float_to_half(float f) noexcept;

}  // namespace quasi::io
