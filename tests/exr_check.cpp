// exr_check.cpp - drives quasi_gb300/host/exr_writer.cpp for tests/test_exr.py (no GPU).
//   exr_check half IN.f32 OUT.u16                    float -> half conversion
//   exr_check rgba W H IN.f32 OUT.exr                 write_exr(Q_readback_result), RGBA input
//   exr_check aov W H B.f32 A.f32 N.f32 D.f32 OUT.exr  write_exr(Q_readback_aov_result); "-" = absent
//   exr_check invalid OUT.exr                         prints the error of each invalid input
#include "exr_writer.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

namespace {

std::vector<float> read_f32(const std::string& path) {
    std::vector<float> v;
    if (path == "-") return v;
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    const auto n = static_cast<size_t>(in.tellg());
    v.resize(n / 4);
    in.seekg(0);
    in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n));
    return v;
}

int report(const std::expected<void, quasi::io::exr_error>& r) {
    if (r) return 0;
    std::printf("%s\n", quasi::io::to_string(r.error()));
    return 3;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 1;
    const std::string mode = argv[1];
    if (mode == "half" && argc == 4) {
        const std::vector<float> in = read_f32(argv[2]);
        std::vector<uint16_t> out(in.size());
        for (size_t i = 0; i < in.size(); ++i) out[i] = quasi::io::float_to_half(in[i]);
        std::ofstream(argv[3], std::ios::binary)
            .write(reinterpret_cast<const char*>(out.data()), static_cast<std::streamsize>(2 * out.size()));
        return 0;
    }
    if (mode == "rgba" && argc == 6) {
        std::vector<float> px = read_f32(argv[4]);
        Q_readback_result r{px.data(), static_cast<uint32_t>(std::atoi(argv[2])),
                            static_cast<uint32_t>(std::atoi(argv[3])), 4};
        return report(quasi::io::write_exr(argv[5], r));
    }
    if (mode == "aov" && argc == 9) {
        const uint32_t w = static_cast<uint32_t>(std::atoi(argv[2])), h = static_cast<uint32_t>(std::atoi(argv[3]));
        std::vector<float> b[4];
        Q_readback_aov_result r{};
        for (int k = 0; k < 4; ++k) {
            b[k] = read_f32(argv[4 + k]);
            if (!b[k].empty()) r.buffers[k] = Q_aov_buffer{b[k].data(), w, h, 4};
        }
        return report(quasi::io::write_exr(argv[8], r));
    }
    if (mode == "invalid" && argc == 3) {
        float px[4] = {1, 2, 3, 4};
        report(quasi::io::write_exr(argv[2], Q_readback_result{nullptr, 1, 1, 4}));
        report(quasi::io::write_exr(argv[2], Q_readback_result{px, 0, 1, 4}));
        report(quasi::io::write_exr(argv[2], Q_readback_aov_result{}));
        Q_readback_aov_result mismatch{};
        mismatch.buffers[0] = Q_aov_buffer{px, 1, 1, 4};
        mismatch.buffers[1] = Q_aov_buffer{px, 2, 1, 4};
        report(quasi::io::write_exr(argv[2], mismatch));
        // a directory that cannot be created: a path below a regular file
        const std::string file = std::string(argv[2]) + ".file";
        std::ofstream(file) << "x";
        report(quasi::io::write_exr(file + "/sub/out.exr", Q_readback_result{px, 1, 1, 4}));
        std::printf("%s\n", quasi::io::make_timestamped_path("dir").string().c_str());
        return 0;
    }
    return 1;
}
