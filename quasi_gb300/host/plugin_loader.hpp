// plugin_loader.hpp - the headless host's plugin loader: dlopen + symbol resolution + ABI
// check + create, with the reference loader's behaviour (src/quasi/plugin/loader.hpp:65-137,
// dynamic_library.hpp): the six required Q_plugin_* symbols (symbol_not_found), an ABI
// version in 1..3 (abi_mismatch), the optional v2/v3 readback symbols, and
// Q_plugin_create returning NULL (create_failed). Reload follows manager.hpp:209-330:
// destroy -> dlclose -> copy the library to a temporary path -> dlopen -> create.
#pragma once

#include "quasi_cuda.h"

#include <dlfcn.h>

#include <cstdint>
#include <filesystem>
#include <string>
#include <system_error>
#include <unistd.h>

namespace quasi::host {

enum class load_error { none, file_not_found, load_failed, symbol_not_found, abi_mismatch, create_failed };

inline const char* to_string(load_error e) {
    switch (e) {
        case load_error::none: return "ok";
        case load_error::file_not_found: return "file_not_found";
        case load_error::load_failed: return "load_failed";
        case load_error::symbol_not_found: return "symbol_not_found";
        case load_error::abi_mismatch: return "abi_mismatch";
        case load_error::create_failed: return "create_failed";
    }
    return "unknown";
}

class plugin {
public:
    plugin() = default;
    ~plugin() { unload(); }
    plugin(const plugin&) = delete;
    plugin& operator=(const plugin&) = delete;

    // Loads `path` (copied to a private temporary file first when `copy` is set, as the
    // reference manager does so the original can be rebuilt while loaded) and creates an
    // instance with `ctx`.
    load_error load(const std::filesystem::path& path, Q_plugin_context* ctx, bool copy) {
        unload();
        if (!std::filesystem::exists(path)) return load_error::file_not_found;
        std::filesystem::path open_path = path;
        if (copy) {
            static int counter = 0;
            open_path = std::filesystem::temp_directory_path() /
                        ("quasi_plugin_" + std::to_string(::getpid()) + "_" + std::to_string(counter++) + ".so");
            std::error_code ec;
            std::filesystem::copy_file(path, open_path, std::filesystem::copy_options::overwrite_existing, ec);
            if (ec) return load_error::load_failed;
            temp_ = open_path;
        }
        lib_ = ::dlopen(open_path.c_str(), RTLD_NOW | RTLD_LOCAL);
        if (!lib_) {
            error_ = ::dlerror();
            return load_error::load_failed;
        }
        if (!sym(abi_version, "Q_plugin_abi_version") || !sym(get_info, "Q_plugin_get_info") ||
            !sym(create, "Q_plugin_create") || !sym(destroy, "Q_plugin_destroy") ||
            !sym(update, "Q_plugin_update") || !sym(render, "Q_plugin_render"))
            return fail(load_error::symbol_not_found);
        abi = abi_version();
        if (abi < 1 || abi > 3) return fail(load_error::abi_mismatch);
        sym(readback, "Q_plugin_readback");
        sym(readback_free, "Q_plugin_readback_free");
        sym(readback_aov, "Q_plugin_readback_aov");
        sym(readback_aov_free, "Q_plugin_readback_aov_free");
        handle = create(ctx);
        if (!handle) return fail(load_error::create_failed);
        return load_error::none;
    }

    void unload() {
        if (handle && destroy) destroy(handle);
        handle = nullptr;
        if (lib_) ::dlclose(lib_);
        lib_ = nullptr;
        if (!temp_.empty()) {
            std::error_code ec;
            std::filesystem::remove(temp_, ec);
            temp_.clear();
        }
        abi_version = nullptr;
        get_info = nullptr;
        create = nullptr;
        destroy = nullptr;
        update = nullptr;
        render = nullptr;
        readback = nullptr;
        readback_free = nullptr;
        readback_aov = nullptr;
        readback_aov_free = nullptr;
    }

    // Optional extension symbol (NULL when absent).
    template <class F> F extension(const char* name) const {
        return lib_ ? reinterpret_cast<F>(::dlsym(lib_, name)) : nullptr;
    }

    const std::string& error() const { return error_; }

    uint32_t (*abi_version)() = nullptr;
    Q_plugin_info (*get_info)() = nullptr;
    Q_plugin_handle* (*create)(Q_plugin_context*) = nullptr;
    void (*destroy)(Q_plugin_handle*) = nullptr;
    void (*update)(Q_plugin_handle*, float) = nullptr;
    void (*render)(Q_plugin_handle*, Q_render_frame*) = nullptr;
    Q_readback_result (*readback)(Q_plugin_handle*) = nullptr;
    void (*readback_free)(Q_readback_result*) = nullptr;
    Q_readback_aov_result (*readback_aov)(Q_plugin_handle*) = nullptr;
    void (*readback_aov_free)(Q_readback_aov_result*) = nullptr;
    Q_plugin_handle* handle = nullptr;
    uint32_t abi = 0;

private:
    template <class F> bool sym(F& fn, const char* name) {
        fn = reinterpret_cast<F>(::dlsym(lib_, name));
        return fn != nullptr;
    }
    load_error fail(load_error e) {
        if (lib_) ::dlclose(lib_);
        lib_ = nullptr;
        handle = nullptr;
        return e;
    }

    void* lib_ = nullptr;
    std::filesystem::path temp_;
    std::string error_;
};

}  // namespace quasi::host
