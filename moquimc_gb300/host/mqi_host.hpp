// Host pieces shared by the C++ drivers over the C ABI (phantom_env_main.cpp, tps_env_main.cpp):
// moqui's input-file and command-line readers, the coordinate-transform rotations, grid edges, the
// volume writers.
#pragma once

#include <array>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <strings.h>

#include "mqi_gpu.h"

namespace mqi_host
{

/// White space trimmed as moqui's trim_copy trims it (moqui/base/mqi_utils.hpp:22-36): space,
/// \f, \n, \r, \t, \v (its delimiter literal ends at an embedded NUL).  moqui throws on a string
/// of white space only; here it trims to "".
inline std::string
trim(const std::string& s) {
    const char*  ws = " \f\n\r\t\v";
    const size_t a = s.find_first_not_of(ws), b = s.find_last_not_of(ws);
    return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

/// mqi::file_parser (moqui/base/mqi_file_handler.hpp:220-420): "Key value" lines; '#' starts a
/// comment line or ends a line; a key is the text before the line's first space and matches
/// case-insensitively; the first matching line wins; numbers are read with atof / atoi, a
/// missing key's default is written with std::to_string first (so a float default keeps six
/// decimals).  moqui's reader throws on a line of white space only, on a value of white space
/// only and on an empty item of a list; here the line is skipped, the value reads as "" and the
/// item is left out.
class InputFile
{
public:
    explicit InputFile(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw std::runtime_error("Cannot open input parameter file.");
        std::string line;
        while (std::getline(f, line)) {
            if (line.empty()) continue;
            line = trim(line);
            if (line.empty() || line[0] == '#') continue;
            const size_t c = line.find('#');
            if (c != std::string::npos) line = line.substr(0, c);
            lines_.push_back(line);
        }
    }
    std::string
    get_string(const std::string& key, const std::string& dflt) const {
        for (const auto& l : lines_) {
            const size_t pos = l.find(' ');
            if (pos != std::string::npos && strcasecmp(trim(l.substr(0, pos)).c_str(), key.c_str()) == 0)
                return trim(l.substr(pos + 1));
        }
        return dflt;
    }
    std::vector<std::string>
    get_vector(const std::string& key, char sep) const {
        std::vector<std::string> out;
        std::stringstream ss(get_string(key, ""));
        std::string t;
        while (std::getline(ss, t, sep))
            if (!trim(t).empty()) out.push_back(trim(t));
        return out;
    }
    float get_float(const std::string& k, float d) const { return std::atof(get_string(k, std::to_string(d)).c_str()); }
    int get_int(const std::string& k, int d) const { return std::atoi(get_string(k, std::to_string(d)).c_str()); }
    bool
    get_bool(const std::string& k, bool d) const {
        const std::string t = get_string(k, std::to_string(d));
        return strcasecmp(t.c_str(), "true") == 0 || std::atoi(t.c_str()) != 0;
    }

private:
    std::vector<std::string> lines_;
};

/// moqui's cli: "--name v1 v2 ..." (moqui/base/mqi_cli.hpp).
class Cli
{
public:
    Cli(int argc, char** argv) {
        std::string key;
        for (int i = 1; i < argc; ++i) {
            const std::string a = argv[i];
            if (a.size() > 2 && a[0] == '-' && a[1] == '-' && !is_number(a)) {
                key = a;
                opts_[key];
            } else if (!key.empty()) {
                opts_[key].push_back(a);
            } else {
                throw std::runtime_error("unexpected argument " + a);
            }
        }
    }
    const std::vector<std::string>&
    operator[](const std::string& k) const {
        static const std::vector<std::string> none;
        auto it = opts_.find(k);
        return it == opts_.end() ? none : it->second;
    }

private:
    static bool
    is_number(const std::string& s) {
        char* end = nullptr;
        std::strtod(s.c_str(), &end);
        return end && *end == '\0';
    }
    std::map<std::string, std::vector<std::string>> opts_;
};

struct Mat3 {
    float m[9] = { 1, 0, 0, 0, 1, 0, 0, 0, 1 };
};

/// mat3x3<float>(a, b, c): identity, then rotations about x, y and z in that order, each applied
/// as the reference's rotate_x/_y/_z updates (moqui/base/mqi_matrix.hpp:69-76, 213-272).
inline Mat3
euler(float a, float b, float c) {
    Mat3 r;
    float& xx = r.m[0]; float& xy = r.m[1]; float& xz = r.m[2];
    float& yx = r.m[3]; float& yy = r.m[4]; float& yz = r.m[5];
    float& zx = r.m[6]; float& zy = r.m[7]; float& zz = r.m[8];
    if (a != 0) {
        const float c1 = std::cos(a), s1 = std::sin(a);
        const float x1 = yx, y1 = yy, z1 = yz;
        yx = c1 * x1 - s1 * zx; yy = c1 * y1 - s1 * zy; yz = c1 * z1 - s1 * zz;
        zx = s1 * x1 + c1 * zx; zy = s1 * y1 + c1 * zy; zz = s1 * z1 + c1 * zz;
    }
    if (b != 0) {
        const float c1 = std::cos(b), s1 = std::sin(b);
        const float x1 = zx, y1 = zy, z1 = zz;
        zx = c1 * x1 - s1 * xx; zy = c1 * y1 - s1 * xy; zz = c1 * z1 - s1 * xz;
        xx = s1 * x1 + c1 * xx; xy = s1 * y1 + c1 * xy; xz = s1 * z1 + c1 * xz;
    }
    if (c != 0) {
        const float c1 = std::cos(c), s1 = std::sin(c);
        const float x1 = xx, y1 = xy, z1 = xz;
        xx = c1 * x1 - s1 * yx; xy = c1 * y1 - s1 * yy; xz = c1 * z1 - s1 * yz;
        yx = s1 * x1 + c1 * yx; yy = s1 * y1 + c1 * yy; yz = s1 * z1 + c1 * yz;
    }
    return r;
}

inline Mat3
mul(const Mat3& a, const Mat3& b) {
    Mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}

/// coordinate_transform: rotation = iec2dicom * couch * gantry * collimator
/// (moqui/base/mqi_coordinate_transform.hpp:52-58).
inline Mat3
beam_rotation(const std::array<float, 4>& ang) {
    const float d2r = (float) (3.14159265358979323846 / 180.0);   // coordinate_transform::deg2rad
    const Mat3 col = euler(0, 0, ang[0] * d2r);
    const Mat3 gan = euler(0, ang[1] * d2r, 0);
    const Mat3 cou = euler(0, 0, ang[2] * d2r);
    const Mat3 iec = euler(ang[3] * d2r, 0, 0);
    return mul(mul(mul(iec, cou), gan), col);
}

/// grid3d's uniform edges from phantom_env::setup_world's corners (mqi_phantom_env.hpp:256-264):
/// corners pos -/+ 0.5 l in double stored as float, then edge_i = min + i * ((max - min) / n).
inline std::vector<float>
edges(float pos, float len, int n) {
    const float lo = (float) (pos - 0.5 * len);
    const float hi = (float) (pos + 0.5 * len);
    const float d  = (hi - lo) / (float) n;
    std::vector<float> e(n + 1);
    for (int i = 0; i <= n; ++i) e[i] = lo + (float) i * d;
    return e;
}

inline float
to_f(const std::vector<std::string>& v, size_t i, float dflt) {
    return v.size() > i ? std::stof(v[i]) : dflt;
}

/// save_to_bin / save_to_mhd / save_to_mha (moqui/base/mqi_io.hpp:166-183, 493-583): the volume
/// times `scale` in FP64, with the reference's header lines (its .mhd writes TransformMatrix,
/// Offset and CenterOfRotation without '=').
inline void
write_outputs(const std::string& dir, const std::string& name, const std::string& fmt, std::vector<double> d,
              double scale, const std::vector<float>& xe, const std::vector<float>& ye, const std::vector<float>& ze) {
    for (double& x : d) x *= scale;
    const int   nx = (int) xe.size() - 1, ny = (int) ye.size() - 1, nz = (int) ze.size() - 1;
    const float dx = xe[1] - xe[0], dy = ye[1] - ye[0], dz = ze[1] - ze[0];
    const float x0 = xe[0] + dx * 0.5f, y0 = ye[0] + dy * 0.5f, z0 = ze[0] + dz * 0.5f;
    if (fmt == "mha") {
        std::ofstream f(dir + "/" + name + ".mha", std::ios::binary);
        f << "ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
          << "CompressedData = False\nTransformMatrix = 1 0 0 0 1 0 0 0 1\n"
          << "Origin = " << std::setprecision(9) << x0 << " " << y0 << " " << z0 << "\n"
          << "CenterOfRotation = 0 0 0\nAnatomicOrientation = RAI\n"
          << "DimSize = " << nx << " " << ny << " " << nz << "\nElementType = MET_DOUBLE\nHeaderSize = -1\n"
          << "ElementSpacing = " << std::setprecision(9) << dx << " " << dy << " " << dz << "\n"
          << "ElementDataFile = LOCAL\n";
        f.write(reinterpret_cast<const char*>(d.data()), d.size() * sizeof(double));
        if (!f) throw std::runtime_error("cannot write " + dir + "/" + name + ".mha");
        return;
    }
    if (fmt == "mhd") {
        std::ofstream h(dir + "/" + name + ".mhd");
        h << "ObjectType = Image\nNDims = 3\nBinaryData = True\nBinaryDataByteOrderMSB = False\n"
          << "CompressedData = False\nTransformMatrix 1 0 0 0 1 0 0 0 1\n"
          << "Offset " << x0 << " " << y0 << " " << z0 << "\nCenterOfRotation 0 0 0\n"
          << "AnatomicOrientation = RAI\nDimSize = " << nx << " " << ny << " " << nz << "\n"
          << "ElementType = MET_DOUBLE\nElementSpacing = " << dx << " " << dy << " " << dz << "\n"
          << "ElementDataFile = " << name << ".raw\n";
        if (!h) throw std::runtime_error("cannot write " + dir + "/" + name + ".mhd");
    }
    std::ofstream r(dir + "/" + name + ".raw", std::ios::binary);
    r.write(reinterpret_cast<const char*>(d.data()), d.size() * sizeof(double));
    if (!r) throw std::runtime_error("cannot write " + dir + "/" + name + ".raw");
}

/// CRC-32 of the zip format (IEEE 802.3 polynomial, reflected: 0xEDB88320), continued from `crc`.
inline uint32_t
crc32_update(uint32_t crc, const void* data, size_t n) {
    static const std::array<uint32_t, 256> table = [] {
        std::array<uint32_t, 256> t{};
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    const unsigned char* p = static_cast<const unsigned char*>(data);
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

/// One member of an npz file: an .npy array (format 1.0) with its dtype descriptor ("<u4",
/// "<f8", "|S3") and shape tuple ("(12,)", "()").
struct NpzArray {
    std::string name;
    std::string descr;
    std::string shape;
    const void* data;
    size_t      bytes;
};

/// mqi::io::save_npz (moqui/base/mqi_sparse_io.hpp:167-399): the arrays as stored (uncompressed)
/// members of a zip archive, in the given order, byte for byte as the reference writes numeric
/// members: the .npy header dictionary padded with spaces until 10 + its length is a multiple of
/// 16 (a full 16 when it already is), then a newline; zero modification time and date; version 20.
/// Like the reference's writer it uses 32-bit zip sizes and offsets; a file past 4 GiB raises
/// instead of wrapping.  One member differs on purpose: a string ("format", "csr") is written as
/// its bytes, where the reference writes sizeof(std::string) bytes per character from the string's
/// buffer (mqi_sparse_io.hpp:241-276), i.e. whatever memory follows the three characters.
inline void
write_npz(const std::string& path, const std::vector<NpzArray>& arrays) {
    auto u16 = [](std::string& s, uint32_t v) { s.push_back((char) (v & 0xFF)); s.push_back((char) ((v >> 8) & 0xFF)); };
    auto u32 = [&](std::string& s, uint32_t v) { u16(s, v & 0xFFFF); u16(s, v >> 16); };
    std::ofstream f(path, std::ios::binary);
    std::string   central;
    uint64_t      offset = 0;
    for (const auto& a : arrays) {
        std::string dict = "{'descr': '" + a.descr + "', 'fortran_order': False, 'shape': " + a.shape + ", }";
        dict.append(16 - (10 + dict.size()) % 16, ' ');
        dict.push_back('\n');
        std::string head("\x93NUMPY\x01", 7);
        head.push_back('\0');
        u16(head, (uint32_t) dict.size());
        head += dict;
        const uint64_t size = head.size() + (uint64_t) a.bytes;
        const std::string fname = a.name + ".npy";
        if (size > 0xFFFFFFFFull || offset + size + 30 + fname.size() > 0xFFFFFFFFull)
            throw std::runtime_error(path + ": npz members past 4 GiB need zip64, which is not written");
        const uint32_t crc = crc32_update(crc32_update(0, head.data(), head.size()), a.data, a.bytes);
        std::string rec;   // the fields the local and central headers share
        u16(rec, 20); u16(rec, 0); u16(rec, 0);            // version needed, flags, stored
        u16(rec, 0); u16(rec, 0);                           // modification time and date: 0
        u32(rec, crc); u32(rec, (uint32_t) size); u32(rec, (uint32_t) size);
        u16(rec, (uint32_t) fname.size()); u16(rec, 0);     // name length, no extra field
        std::string local("PK\x03\x04", 4);
        local += rec + fname;
        f.write(local.data(), (std::streamsize) local.size());
        f.write(head.data(), (std::streamsize) head.size());
        f.write(static_cast<const char*>(a.data), (std::streamsize) a.bytes);
        std::string cent("PK\x01\x02", 4);
        u16(cent, 20);
        cent += rec;
        u16(cent, 0); u16(cent, 0); u16(cent, 0); u32(cent, 0);   // comment, disk, attributes
        u32(cent, (uint32_t) offset);
        central += cent + fname;
        offset += local.size() + size;
    }
    if (offset + central.size() > 0xFFFFFFFFull)
        throw std::runtime_error(path + ": npz past 4 GiB needs zip64, which is not written");
    std::string end("PK\x05\x06", 4);
    u16(end, 0); u16(end, 0); u16(end, (uint32_t) arrays.size()); u16(end, (uint32_t) arrays.size());
    u32(end, (uint32_t) central.size()); u32(end, (uint32_t) offset); u16(end, 0);
    f.write(central.data(), (std::streamsize) central.size());
    f.write(end.data(), (std::streamsize) end.size());
    if (!f) throw std::runtime_error("cannot write " + path);
}

inline void
check(int rc, mqi_ctx* ctx, const char* what) {
    if (rc != MQI_OK) throw std::runtime_error(std::string(what) + ": " + mqi_last_error(ctx));
}

}   // namespace mqi_host
