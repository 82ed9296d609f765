#include "io.hpp"

#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <stdexcept>

namespace {

std::vector<float> read_floats(const std::string& path)
{
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (f == nullptr) {
        throw std::runtime_error(path + ": cannot open");
    }
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (bytes < 0 || bytes % 4 != 0) {
        std::fclose(f);
        throw std::runtime_error(path + ": size is not a whole number of float32 values");
    }
    std::vector<float> v(static_cast<std::size_t>(bytes) / 4);
    const std::size_t got = v.empty() ? 0 : std::fread(v.data(), 4, v.size(), f);
    std::fclose(f);
    if (got != v.size()) {
        throw std::runtime_error(path + ": short read");
    }
    return v;
}

void write_bytes(const std::string& path, const void* data, std::size_t bytes)
{
    std::FILE* f = std::fopen(path.c_str(), "wb");
    if (f == nullptr) {
        throw std::runtime_error(path + ": cannot create");
    }
    const std::size_t put = bytes == 0 ? 0 : std::fwrite(data, 1, bytes, f);
    std::fclose(f);
    if (put != bytes) {
        throw std::runtime_error(path + ": short write");
    }
}

}  // namespace

std::vector<cf32> read_cf32(const std::string& path)
{
    const std::vector<float> v = read_floats(path);
    if (v.size() % 2 != 0) {
        throw std::runtime_error(path + ": odd number of float32 values, not interleaved IQ");
    }
    std::vector<cf32> x(v.size() / 2);
    for (std::size_t i = 0; i < x.size(); ++i) {
        x[i] = cf32{v[2 * i], v[2 * i + 1]};
    }
    return x;
}

std::vector<float> read_f32(const std::string& path) { return read_floats(path); }

void write_cf32(const std::string& path, const std::vector<cf32>& x)
{
    write_bytes(path, x.data(), x.size() * sizeof(cf32));
}

void write_f32(const std::string& path, const std::vector<float>& x)
{
    write_bytes(path, x.data(), x.size() * sizeof(float));
}

double sample_rate(const std::string& path)
{
    const std::string meta = std::filesystem::path(path).replace_extension(".json").string();
    std::ifstream in(meta);
    if (!in) {
        return 0.0;
    }
    const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    const std::string key = "\"sample_rate\"";
    const std::size_t at = text.find(key);
    if (at == std::string::npos) {
        return 0.0;
    }
    const std::size_t colon = text.find(':', at + key.size());
    return colon == std::string::npos ? 0.0 : std::strtod(text.c_str() + colon + 1, nullptr);
}
