#include "io.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <stdexcept>

namespace {

// The whole file, whose size must be a multiple of `unit` bytes (`what` names the unit).
std::vector<std::uint8_t> read_file(const std::string& path, std::size_t unit, const char* what)
{
    std::FILE* f = std::fopen(path.c_str(), "rb");
    if (f == nullptr) {
        throw std::runtime_error(path + ": cannot open");
    }
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (bytes < 0 || static_cast<std::size_t>(bytes) % unit != 0) {
        std::fclose(f);
        throw std::runtime_error(path + ": size is not a whole number of " + what);
    }
    std::vector<std::uint8_t> v(static_cast<std::size_t>(bytes));
    const std::size_t got = v.empty() ? 0 : std::fread(v.data(), 1, v.size(), f);
    std::fclose(f);
    if (got != v.size()) {
        throw std::runtime_error(path + ": short read");
    }
    return v;
}

std::vector<float> read_floats(const std::string& path)
{
    const std::vector<std::uint8_t> raw = read_file(path, 4, "float32 values");
    std::vector<float> v(raw.size() / 4);
    if (!v.empty()) {
        std::memcpy(v.data(), raw.data(), raw.size());
    }
    return v;
}

std::string read_text(const std::string& path)
{
    std::ifstream in(path);
    if (!in) {
        throw std::runtime_error(path + ": cannot open");
    }
    return std::string((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

bool has_suffix(const std::string& s, const char* suffix)
{
    const std::size_t k = std::strlen(suffix);
    return s.size() >= k && s.compare(s.size() - k, k, suffix) == 0;
}

// NAME for NAME.sigmf-meta or NAME.sigmf-data (both suffixes have the same length).
std::string sigmf_stem(const std::string& path)
{
    return path.substr(0, path.size() - std::strlen(".sigmf-meta"));
}

// The value of the first "key": member in a JSON text, unquoted: a string's characters, or a
// number's or literal's text. Empty when the key is absent. Enough for the flat "global"
// fields of a SigMF header (no escapes in the values read here).
std::string json_value(const std::string& text, const std::string& key)
{
    const std::string quoted = "\"" + key + "\"";
    std::size_t at = text.find(quoted);
    while (at != std::string::npos) {
        std::size_t i = at + quoted.size();
        while (i < text.size() && std::strchr(" \t\r\n", text[i]) != nullptr) {
            ++i;
        }
        if (i < text.size() && text[i] == ':') {
            ++i;
            while (i < text.size() && std::strchr(" \t\r\n", text[i]) != nullptr) {
                ++i;
            }
            if (i < text.size() && text[i] == '"') {
                const std::size_t end = text.find('"', i + 1);
                return text.substr(i + 1, end == std::string::npos ? std::string::npos
                                                                    : end - i - 1);
            }
            const std::size_t end = text.find_first_of(",}] \t\r\n", i);
            return text.substr(i, end == std::string::npos ? std::string::npos : end - i);
        }
        at = text.find(quoted, at + 1);  // the key's text inside another string: keep looking
    }
    return std::string();
}

std::size_t format_bytes(SampleFormat f)
{
    return f == SampleFormat::Cf32 ? 8 : f == SampleFormat::Ci16 ? 4 : 2;
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

bool is_sigmf(const std::string& path)
{
    return has_suffix(path, ".sigmf-meta") || has_suffix(path, ".sigmf-data");
}

SampleFormat sample_format(const std::string& path)
{
    if (!is_sigmf(path)) {
        return SampleFormat::Cf32;
    }
    const std::string meta_path = sigmf_stem(path) + ".sigmf-meta";
    const std::string meta = read_text(meta_path);
    const std::string channels = json_value(meta, "core:num_channels");
    if (!channels.empty() && std::atoi(channels.c_str()) != 1) {
        throw std::runtime_error(meta_path + ": " + channels +
                                 " channels; only single-channel recordings are supported");
    }
    const std::string type = json_value(meta, "core:datatype");
    if (type == "cf32_le") {
        return SampleFormat::Cf32;
    }
    if (type == "ci16_le") {
        return SampleFormat::Ci16;
    }
    if (type == "ci8" || type == "ci8_le") {
        return SampleFormat::Ci8;
    }
    throw std::runtime_error(meta_path + ": core:datatype '" + type +
                             "' is not supported (cf32_le, ci16_le, ci8)");
}

StoredSamples read_stored(const std::string& path)
{
    StoredSamples s;
    s.format = sample_format(path);
    const std::string data = is_sigmf(path) ? sigmf_stem(path) + ".sigmf-data" : path;
    const char* what = s.format == SampleFormat::Cf32   ? "interleaved float32 I/Q samples"
                       : s.format == SampleFormat::Ci16 ? "interleaved int16 I/Q samples"
                                                        : "interleaved int8 I/Q samples";
    s.bytes = read_file(data, format_bytes(s.format), what);
    s.count = s.bytes.size() / format_bytes(s.format);
    return s;
}

std::vector<cf32> to_cf32(const StoredSamples& s)
{
    std::vector<cf32> x(s.count);
    if (s.count == 0) {
        return x;
    }
    if (s.format == SampleFormat::Cf32) {
        std::memcpy(x.data(), s.bytes.data(), s.count * sizeof(cf32));
        return x;
    }
    for (std::size_t i = 0; i < s.count; ++i) {
        // Little-endian components, sign-extended explicitly (no reliance on char's sign).
        if (s.format == SampleFormat::Ci16) {
            const std::uint8_t* p = s.bytes.data() + 4 * i;
            const int re = static_cast<std::int16_t>(static_cast<std::uint16_t>(p[0] | p[1] << 8));
            const int im = static_cast<std::int16_t>(static_cast<std::uint16_t>(p[2] | p[3] << 8));
            x[i] = cf32{static_cast<float>(re) * (1.0f / 32768.0f),
                        static_cast<float>(im) * (1.0f / 32768.0f)};
        } else {
            const std::uint8_t* p = s.bytes.data() + 2 * i;
            const int re = static_cast<std::int8_t>(p[0]);
            const int im = static_cast<std::int8_t>(p[1]);
            x[i] = cf32{static_cast<float>(re) * (1.0f / 128.0f),
                        static_cast<float>(im) * (1.0f / 128.0f)};
        }
    }
    return x;
}

std::vector<cf32> read_cf32(const std::string& path)
{
    return to_cf32(read_stored(path));
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
    std::string meta;
    std::string key;
    if (is_sigmf(path)) {
        meta = sigmf_stem(path) + ".sigmf-meta";
        key = "core:sample_rate";
    } else {
        meta = std::filesystem::path(path).replace_extension(".json").string();
        key = "sample_rate";
        if (!std::filesystem::exists(meta)) {
            return 0.0;
        }
    }
    const std::string value = json_value(read_text(meta), key);
    return value.empty() ? 0.0 : std::strtod(value.c_str(), nullptr);
}
