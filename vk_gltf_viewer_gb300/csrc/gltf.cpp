// glTF 2.0 import into the renderer's layout: the part of
// src/vk_gltf_viewer/assets.cpp (loadGltf :526-552, processPrimitive
// :288-430, MaterialLoadTask :474-518) and World::addAsset (world.cpp:9-80)
// that turns a .gltf / .glb file into primitives with meshlets, materials,
// a node tree and animation samplers.  The reference parses with fastgltf,
// which is absent from its tree; this is an own JSON and GLB reader that
// follows the glTF 2.0 specification for what the reference asks fastgltf
// for: GenerateMeshIndices, DecomposeNodeMatrices, KHR_mesh_quantization and
// KHR_texture_transform, and EXT_meshopt_compression buffer views, decoded
// by meshopt.cpp (meshoptimizer's codecs are absent too).  Host code, run
// once per asset.
#include "vkgv.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <new>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ------------------------------------------------------------------ JSON

struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double n = 0.0;
    std::string s;
    std::vector<JValue> items;
    std::vector<std::pair<std::string, JValue>> members;

    const JValue* get(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
    bool is_num() const { return kind == Number; }
};

class JsonParser {
public:
    JsonParser(const char* p, size_t n) : begin_(p), p_(p), end_(p + n) {}

    bool parse(JValue& out, std::string& err) {
        skip();
        if (!value(out, 0)) {
            err = "JSON: " + err_ + " at byte " + std::to_string(pos());
            return false;
        }
        skip();
        if (p_ != end_) {
            err = "JSON: trailing characters at byte " + std::to_string(pos());
            return false;
        }
        return true;
    }

private:
    const char* begin_;
    const char* p_;
    const char* end_;
    std::string err_;

    size_t pos() const { return size_t(p_ - begin_); }
    void skip() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool fail(const char* m) {
        err_ = m;
        return false;
    }
    bool literal(const char* word) {
        size_t n = std::strlen(word);
        if (size_t(end_ - p_) < n || std::memcmp(p_, word, n) != 0) return fail("bad literal");
        p_ += n;
        return true;
    }

    bool value(JValue& v, int depth) {
        if (depth > 128) return fail("nesting too deep");
        if (p_ >= end_) return fail("unexpected end");
        switch (*p_) {
            case '{': return object(v, depth);
            case '[': return array(v, depth);
            case '"': v.kind = JValue::String; return string(v.s);
            case 't': v.kind = JValue::Bool; v.b = true; return literal("true");
            case 'f': v.kind = JValue::Bool; v.b = false; return literal("false");
            case 'n': v.kind = JValue::Null; return literal("null");
            default: return number(v);
        }
    }

    bool object(JValue& v, int depth) {
        v.kind = JValue::Object;
        ++p_;
        skip();
        if (p_ < end_ && *p_ == '}') {
            ++p_;
            return true;
        }
        while (true) {
            skip();
            if (p_ >= end_ || *p_ != '"') return fail("expected a member name");
            std::string key;
            if (!string(key)) return false;
            skip();
            if (p_ >= end_ || *p_ != ':') return fail("expected ':'");
            ++p_;
            skip();
            v.members.emplace_back(std::move(key), JValue{});
            if (!value(v.members.back().second, depth + 1)) return false;
            skip();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == '}') {
                ++p_;
                return true;
            }
            return fail("expected ',' or '}'");
        }
    }

    bool array(JValue& v, int depth) {
        v.kind = JValue::Array;
        ++p_;
        skip();
        if (p_ < end_ && *p_ == ']') {
            ++p_;
            return true;
        }
        while (true) {
            skip();
            v.items.emplace_back();
            if (!value(v.items.back(), depth + 1)) return false;
            skip();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == ']') {
                ++p_;
                return true;
            }
            return fail("expected ',' or ']'");
        }
    }

    static void put_utf8(std::string& s, uint32_t c) {
        if (c < 0x80) {
            s += char(c);
        } else if (c < 0x800) {
            s += char(0xC0 | (c >> 6));
            s += char(0x80 | (c & 0x3F));
        } else if (c < 0x10000) {
            s += char(0xE0 | (c >> 12));
            s += char(0x80 | ((c >> 6) & 0x3F));
            s += char(0x80 | (c & 0x3F));
        } else {
            s += char(0xF0 | (c >> 18));
            s += char(0x80 | ((c >> 12) & 0x3F));
            s += char(0x80 | ((c >> 6) & 0x3F));
            s += char(0x80 | (c & 0x3F));
        }
    }

    bool hex4(uint32_t& out) {
        if (end_ - p_ < 4) return fail("short \\u escape");
        out = 0;
        for (int i = 0; i < 4; ++i) {
            char c = *p_++;
            out <<= 4;
            if (c >= '0' && c <= '9') out |= uint32_t(c - '0');
            else if (c >= 'a' && c <= 'f') out |= uint32_t(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') out |= uint32_t(c - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }

    bool string(std::string& s) {
        ++p_;  // opening quote
        while (p_ < end_) {
            char c = *p_++;
            if (c == '"') return true;
            if (static_cast<unsigned char>(c) < 0x20) return fail("control character in string");
            if (c != '\\') {
                s += c;
                continue;
            }
            if (p_ >= end_) break;
            char e = *p_++;
            switch (e) {
                case '"': s += '"'; break;
                case '\\': s += '\\'; break;
                case '/': s += '/'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'n': s += '\n'; break;
                case 'r': s += '\r'; break;
                case 't': s += '\t'; break;
                case 'u': {
                    uint32_t cp;
                    if (!hex4(cp)) return false;
                    if (cp >= 0xD800 && cp < 0xDC00) {  // a surrogate pair
                        uint32_t lo;
                        if (end_ - p_ < 2 || p_[0] != '\\' || p_[1] != 'u') return fail("lone surrogate");
                        p_ += 2;
                        if (!hex4(lo) || lo < 0xDC00 || lo >= 0xE000) return fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    put_utf8(s, cp);
                    break;
                }
                default: return fail("bad escape");
            }
        }
        return fail("unterminated string");
    }

    bool number(JValue& v) {
        const char* start = p_;
        if (p_ < end_ && *p_ == '-') ++p_;
        if (p_ >= end_ || !(*p_ >= '0' && *p_ <= '9')) return fail("bad value");
        while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '+' ||
                             *p_ == '-'))
            ++p_;
        std::string text(start, p_);
        char* stop = nullptr;
        v.kind = JValue::Number;
        v.n = std::strtod(text.c_str(), &stop);
        if (!stop || *stop != '\0') return fail("bad number");
        return true;
    }
};

// --------------------------------------------------------------- helpers

struct ImportError {
    std::string msg;
};

[[noreturn]] void fail(const std::string& m) { throw ImportError{m}; }

double num(const JValue& o, const char* key, double def) {
    const JValue* v = o.get(key);
    if (!v) return def;
    if (!v->is_num()) fail(std::string("'") + key + "' must be a number");
    return v->n;
}

int64_t index_of(const JValue& o, const char* key, int64_t def = -1) {
    const JValue* v = o.get(key);
    if (!v) return def;
    if (!v->is_num() || v->n < 0 || v->n != std::floor(v->n) || v->n > 4294967295.0)
        fail(std::string("'") + key + "' must be a non-negative integer");
    return int64_t(v->n);
}

const JValue& array_of(const JValue& root, const char* key) {
    static const JValue empty = [] {
        JValue v;
        v.kind = JValue::Array;
        return v;
    }();
    const JValue* v = root.get(key);
    if (!v) return empty;
    if (v->kind != JValue::Array) fail(std::string("'") + key + "' must be an array");
    return *v;
}

std::vector<uint8_t> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) fail("cannot open " + path);
    std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return data;
}

std::vector<uint8_t> base64(const std::string& s, size_t start) {
    // built once, thread-safely (a function-local static)
    static const std::array<int8_t, 256> table = [] {
        std::array<int8_t, 256> t;
        t.fill(-1);
        const char* a = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
        for (int i = 0; i < 64; ++i) t[uint8_t(a[i])] = int8_t(i);
        return t;
    }();
    std::vector<uint8_t> out;
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = start; i < s.size(); ++i) {
        uint8_t c = uint8_t(s[i]);
        if (c == '=') break;
        if (table[c] < 0) fail("bad base64 data URI");
        acc = (acc << 6) | uint32_t(table[c]);
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back(uint8_t(acc >> bits));
        }
    }
    return out;
}

std::string percent_decode(const std::string& s) {
    std::string out;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == '%' && i + 2 < s.size()) {
            out += char(std::stoi(s.substr(i + 1, 2), nullptr, 16));
            i += 2;
        } else {
            out += s[i];
        }
    }
    return out;
}

uint32_t component_size(uint32_t ct) {
    switch (ct) {
        case 5120: case 5121: return 1;
        case 5122: case 5123: return 2;
        case 5125: case 5126: return 4;
        default: fail("unknown accessor componentType " + std::to_string(ct));
    }
}

uint32_t type_components(const std::string& t) {
    if (t == "SCALAR") return 1;
    if (t == "VEC2") return 2;
    if (t == "VEC3") return 3;
    if (t == "VEC4") return 4;
    if (t == "MAT2") return 4;
    if (t == "MAT3") return 9;
    if (t == "MAT4") return 16;
    fail("unknown accessor type " + t);
}

// One component as float: the glTF 2.0 rules for normalized integers
// (max(c / (2^(b-1) - 1), -1) signed, c / (2^b - 1) unsigned), plain
// conversion otherwise (KHR_mesh_quantization allows unnormalized integers).
float component_as_float(const uint8_t* p, uint32_t ct, bool normalized) {
    switch (ct) {
        case 5126: {
            float f;
            std::memcpy(&f, p, 4);
            return f;
        }
        case 5120: {
            int8_t c = int8_t(p[0]);
            return normalized ? std::max(float(c) / 127.0f, -1.0f) : float(c);
        }
        case 5121: return normalized ? float(p[0]) / 255.0f : float(p[0]);
        case 5122: {
            int16_t c;
            std::memcpy(&c, p, 2);
            return normalized ? std::max(float(c) / 32767.0f, -1.0f) : float(c);
        }
        case 5123: {
            uint16_t c;
            std::memcpy(&c, p, 2);
            return normalized ? float(c) / 65535.0f : float(c);
        }
        case 5125: {
            uint32_t c;
            std::memcpy(&c, p, 4);
            return normalized ? float(double(c) / 4294967295.0) : float(c);
        }
        default: return 0.0f;
    }
}

uint32_t component_as_index(const uint8_t* p, uint32_t ct) {
    switch (ct) {
        case 5121: return p[0];
        case 5123: {
            uint16_t c;
            std::memcpy(&c, p, 2);
            return c;
        }
        case 5125: {
            uint32_t c;
            std::memcpy(&c, p, 4);
            return c;
        }
        default: fail("index accessors must be UNSIGNED_BYTE, UNSIGNED_SHORT or UNSIGNED_INT");
    }
}

// ------------------------------------------------------------------ asset

struct View {
    const uint8_t* data;  // the view's first byte: in its buffer, or the decoded copy
    size_t length, stride;
};

struct Accessor {
    int64_t view = -1;
    size_t offset = 0, count = 0;
    uint32_t component = 5126, ncomp = 1;
    bool normalized = false;
    const JValue* json = nullptr;
};

// One EXT_meshopt_compression bufferView to decode.
struct CompressedView {
    size_t view;
    const uint8_t* src;
    size_t size, count, stride;
    int mode, filter;
};

int meshopt_enum(const JValue& o, const char* key, const char* def, const char* const* names, int n) {
    const JValue* v = o.get(key);
    if (!v && def) return 0;
    if (!v || v->kind != JValue::String) fail(std::string("EXT_meshopt_compression.") + key + " missing");
    for (int i = 0; i < n; ++i)
        if (v->s == names[i]) return i;
    fail(std::string("EXT_meshopt_compression.") + key + " '" + v->s + "' is not known");
}

}  // namespace

namespace vkgv {
size_t meshopt_threaded_bytes();
int meshopt_decode(void* dst, uint64_t count, uint64_t stride, const void* src, uint64_t size, int mode, int filter,
                   unsigned threads);
}  // namespace vkgv

namespace {

// Decodes the compressed views (assets.cpp:111-166 runs them as a task set
// over the bufferViews): small views in parallel, one thread each, then the
// large ones one at a time with their blocks split over the threads.
void decode_views(const std::vector<CompressedView>& jobs, std::vector<std::vector<uint8_t>>& out) {
    out.resize(jobs.size());
    for (size_t i = 0; i < jobs.size(); ++i) out[i].resize(jobs[i].count * jobs[i].stride);
    const unsigned hw = std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<int> status(jobs.size(), VKGV_OK);
    std::vector<size_t> small, large;
    size_t small_bytes = 0;
    for (size_t i = 0; i < jobs.size(); ++i) {
        if (out[i].size() >= vkgv::meshopt_threaded_bytes()) {
            large.push_back(i);
        } else {
            small.push_back(i);
            small_bytes += out[i].size();
        }
    }
    auto run = [&](size_t i, unsigned threads) {
        const CompressedView& j = jobs[i];
        status[i] = vkgv::meshopt_decode(out[i].data(), j.count, j.stride, j.src, j.size, j.mode, j.filter, threads);
    };
    const size_t threads = small_bytes < (size_t(1) << 20) ? 1 : std::min<size_t>(small.size(), hw);
    if (threads <= 1) {
        for (size_t i : small) run(i, 1);
    } else {
        std::atomic<size_t> next{0};
        std::vector<std::thread> pool;
        for (size_t t = 0; t < threads; ++t)
            pool.emplace_back([&] {
                for (size_t k; (k = next.fetch_add(1)) < small.size();) run(small[k], 1);
            });
        for (auto& th : pool) th.join();
    }
    for (size_t i : large) run(i, hw);
    for (size_t i = 0; i < jobs.size(); ++i) {
        if (status[i] == VKGV_OUT_OF_MEMORY) throw std::bad_alloc();
        if (status[i] != VKGV_OK)
            fail("EXT_meshopt_compression bufferView " + std::to_string(jobs[i].view) + " does not decode");
    }
}

class Reader {
public:
    // placeholder[b]: buffer b is an EXT_meshopt_compression fallback without data
    Reader(const JValue& root, const std::vector<std::vector<uint8_t>>& buffers, const std::vector<bool>& placeholder)
        : root_(root) {
        static const char* const kModes[] = {"ATTRIBUTES", "TRIANGLES", "INDICES"};
        static const char* const kFilters[] = {"NONE", "OCTAHEDRAL", "QUATERNION", "EXPONENTIAL"};
        std::vector<CompressedView> jobs;
        for (const JValue& v : array_of(root, "bufferViews").items) {
            View bv{nullptr, 0, 0};
            const int64_t len = index_of(v, "byteLength");
            if (len < 0) fail("bufferView.byteLength missing");
            bv.stride = size_t(index_of(v, "byteStride", 0));
            const JValue* ext = v.get("extensions");
            const JValue* mc = ext ? ext->get("EXT_meshopt_compression") : nullptr;
            if (mc) {
                CompressedView j;
                j.view = views_.size();
                const int64_t b = index_of(*mc, "buffer"), off = index_of(*mc, "byteOffset", 0);
                const int64_t size = index_of(*mc, "byteLength"), stride = index_of(*mc, "byteStride");
                const int64_t count = index_of(*mc, "count");
                if (b < 0 || size_t(b) >= buffers.size()) fail("EXT_meshopt_compression.buffer out of range");
                if (size < 0 || stride <= 0 || count < 0) fail("EXT_meshopt_compression without byteLength, byteStride or count");
                if (placeholder[size_t(b)]) fail("EXT_meshopt_compression data in a buffer without data");
                if (size_t(off + size) > buffers[size_t(b)].size()) fail("EXT_meshopt_compression data exceeds its buffer");
                j.mode = meshopt_enum(*mc, "mode", nullptr, kModes, 3);
                j.filter = meshopt_enum(*mc, "filter", "NONE", kFilters, 4);
                // a stream holds at most 64 vertices per byte (attributes) or
                // one index per byte (index codecs): larger counts are malformed
                const double most = j.mode == VKGV_MESHOPT_ATTRIBUTES ? 64.0 * double(size) + 256.0 : 3.0 * double(size);
                if (double(count) > most) fail("EXT_meshopt_compression.count exceeds what its data can hold");
                j.src = buffers[size_t(b)].data() + off;
                j.size = size_t(size);
                j.count = size_t(count);
                j.stride = size_t(stride);
                bv.length = j.count * j.stride;
                jobs.push_back(j);
            } else {
                const int64_t b = index_of(v, "buffer");
                if (b < 0 || size_t(b) >= buffers.size()) fail("bufferView.buffer out of range");
                if (placeholder[size_t(b)]) fail("bufferView reads a buffer without data (an EXT_meshopt_compression fallback)");
                const size_t off = size_t(index_of(v, "byteOffset", 0));
                bv.length = size_t(len);
                if (off + bv.length > buffers[size_t(b)].size()) fail("bufferView exceeds its buffer");
                bv.data = buffers[size_t(b)].data() + off;
            }
            views_.push_back(bv);
        }
        decode_views(jobs, decoded_);
        for (size_t i = 0; i < jobs.size(); ++i) views_[jobs[i].view].data = decoded_[i].data();
        for (const JValue& a : array_of(root, "accessors").items) {
            Accessor ac;
            ac.view = index_of(a, "bufferView");
            ac.offset = size_t(index_of(a, "byteOffset", 0));
            const int64_t count = index_of(a, "count");
            if (count < 0) fail("accessor.count missing");
            ac.count = size_t(count);
            ac.component = uint32_t(index_of(a, "componentType"));
            const JValue* t = a.get("type");
            if (!t || t->kind != JValue::String) fail("accessor.type missing");
            ac.ncomp = type_components(t->s);
            const JValue* nz = a.get("normalized");
            ac.normalized = nz && nz->kind == JValue::Bool && nz->b;
            ac.json = &a;
            if (ac.view >= int64_t(views_.size())) fail("accessor.bufferView out of range");
            component_size(ac.component);
            accessors_.push_back(ac);
        }
    }

    const Accessor& accessor(int64_t i) const {
        if (i < 0 || size_t(i) >= accessors_.size()) fail("accessor index out of range");
        return accessors_[size_t(i)];
    }

    // Element k's components as raw bytes (nullptr for an accessor without a
    // bufferView, which reads as zeros).
    template <class F>
    void each_element(const Accessor& a, F&& f) const {
        const uint32_t cs = component_size(a.component);
        const size_t elem = size_t(cs) * a.ncomp;
        if (a.view < 0) {
            std::vector<uint8_t> zero(elem, 0);
            for (size_t k = 0; k < a.count; ++k) f(k, zero.data(), cs);
        } else {
            const View& v = views_[size_t(a.view)];
            const size_t stride = v.stride ? v.stride : elem;
            if (a.count && a.offset + (a.count - 1) * stride + elem > v.length) fail("accessor exceeds its bufferView");
            const uint8_t* base = v.data + a.offset;
            for (size_t k = 0; k < a.count; ++k) f(k, base + k * stride, cs);
        }
    }

    std::vector<float> floats(const Accessor& a) const {
        std::vector<float> out(a.count * a.ncomp);
        each_element(a, [&](size_t k, const uint8_t* p, uint32_t cs) {
            for (uint32_t c = 0; c < a.ncomp; ++c)
                out[k * a.ncomp + c] = component_as_float(p + size_t(c) * cs, a.component, a.normalized);
        });
        apply_sparse(a, [&](size_t k, const uint8_t* p, uint32_t cs) {
            for (uint32_t c = 0; c < a.ncomp; ++c)
                out[k * a.ncomp + c] = component_as_float(p + size_t(c) * cs, a.component, a.normalized);
        });
        return out;
    }

    std::vector<uint32_t> indices(const Accessor& a) const {
        if (a.ncomp != 1) fail("index accessors must be SCALAR");
        std::vector<uint32_t> out(a.count);
        each_element(a, [&](size_t k, const uint8_t* p, uint32_t) { out[k] = component_as_index(p, a.component); });
        apply_sparse(a, [&](size_t k, const uint8_t* p, uint32_t) { out[k] = component_as_index(p, a.component); });
        return out;
    }

private:
    const JValue& root_;
    std::vector<View> views_;
    std::vector<std::vector<uint8_t>> decoded_;  // EXT_meshopt_compression views
    std::vector<Accessor> accessors_;

    // accessor.sparse: values replace the listed elements.
    template <class F>
    void apply_sparse(const Accessor& a, F&& f) const {
        const JValue* sp = a.json->get("sparse");
        if (!sp) return;
        const int64_t scount = index_of(*sp, "count");
        if (scount < 0) fail("sparse.count missing");
        const size_t count = size_t(scount);
        const JValue* ij = sp->get("indices");
        const JValue* vj = sp->get("values");
        if (!ij || !vj) fail("sparse accessor without indices or values");
        const int64_t iv = index_of(*ij, "bufferView"), vv = index_of(*vj, "bufferView");
        if (iv < 0 || vv < 0 || size_t(iv) >= views_.size() || size_t(vv) >= views_.size())
            fail("sparse bufferView out of range");
        const uint32_t ict = uint32_t(index_of(*ij, "componentType"));
        const uint32_t ics = component_size(ict), cs = component_size(a.component);
        const View& I = views_[size_t(iv)];
        const View& V = views_[size_t(vv)];
        const size_t ioff = size_t(index_of(*ij, "byteOffset", 0)), voff = size_t(index_of(*vj, "byteOffset", 0));
        const size_t elem = size_t(cs) * a.ncomp;
        if (ioff + count * ics > I.length || voff + count * elem > V.length) fail("sparse data exceeds its bufferView");
        const uint8_t* ib = I.data + ioff;
        const uint8_t* vb = V.data + voff;
        for (size_t i = 0; i < count; ++i) {
            const uint32_t k = component_as_index(ib + i * ics, ict);
            if (k >= a.count) fail("sparse index out of range");
            f(k, vb + i * elem, cs);
        }
    }
};

// Node matrix -> TRS (fastgltf's DecomposeNodeMatrices, restated): T is
// column 3, S the column lengths (x negated for a mirroring matrix), R the
// quaternion of the normalised rotation (Shepperd's method), in float64.
void decompose(const double m[16], float t[3], float q[4], float s[3]) {
    for (int i = 0; i < 3; ++i) t[i] = float(m[12 + i]);
    double c[3][3], len[3];
    for (int j = 0; j < 3; ++j) {
        len[j] = std::sqrt(m[4 * j] * m[4 * j] + m[4 * j + 1] * m[4 * j + 1] + m[4 * j + 2] * m[4 * j + 2]);
        for (int i = 0; i < 3; ++i) c[j][i] = len[j] > 0 ? m[4 * j + i] / len[j] : 0.0;
    }
    const double det = c[0][0] * (c[1][1] * c[2][2] - c[2][1] * c[1][2]) -
                       c[1][0] * (c[0][1] * c[2][2] - c[2][1] * c[0][2]) +
                       c[2][0] * (c[0][1] * c[1][2] - c[1][1] * c[0][2]);
    if (det < 0) {
        len[0] = -len[0];
        for (int i = 0; i < 3; ++i) c[0][i] = -c[0][i];
    }
    for (int j = 0; j < 3; ++j) s[j] = float(len[j]);
    // R[row][col] = c[col][row]
    const double r00 = c[0][0], r11 = c[1][1], r22 = c[2][2];
    const double tr = r00 + r11 + r22;
    double x, y, z, w;
    if (tr > 0) {
        const double k = 0.5 / std::sqrt(tr + 1.0);
        w = 0.25 / k;
        x = (c[1][2] - c[2][1]) * k;
        y = (c[2][0] - c[0][2]) * k;
        z = (c[0][1] - c[1][0]) * k;
    } else if (r00 > r11 && r00 > r22) {
        const double k = 2.0 * std::sqrt(1.0 + r00 - r11 - r22);
        w = (c[1][2] - c[2][1]) / k;
        x = 0.25 * k;
        y = (c[1][0] + c[0][1]) / k;
        z = (c[2][0] + c[0][2]) / k;
    } else if (r11 > r22) {
        const double k = 2.0 * std::sqrt(1.0 + r11 - r00 - r22);
        w = (c[2][0] - c[0][2]) / k;
        x = (c[1][0] + c[0][1]) / k;
        y = 0.25 * k;
        z = (c[2][1] + c[1][2]) / k;
    } else {
        const double k = 2.0 * std::sqrt(1.0 + r22 - r00 - r11);
        w = (c[0][1] - c[1][0]) / k;
        x = (c[2][0] + c[0][2]) / k;
        y = (c[2][1] + c[1][2]) / k;
        z = 0.25 * k;
    }
    const double n = std::sqrt(x * x + y * y + z * z + w * w);
    q[0] = float(x / n), q[1] = float(y / n), q[2] = float(z / n), q[3] = float(w / n);
}

}  // namespace

struct vkgv_gltf {
    std::vector<vkgv_mesh*> meshes;               // one per primitive
    std::vector<uint32_t> prim_material, prim_mesh;
    std::vector<vkgv_material> materials;
    std::vector<vkgv_node> nodes;
    std::vector<uint32_t> children, roots;
    std::vector<uint32_t> mesh_offsets, mesh_primitives, meshlet_counts;
    std::vector<std::vector<float>> keys;         // per sampler: input then output
    std::vector<vkgv_anim_sampler> samplers;
    std::vector<vkgv_anim_channel> channels;
    uint32_t texture_count = 0, image_count = 0;
    std::vector<std::vector<uint8_t>> texture_images;  // per texture (VKGV_GLTF_IMAGES), may be empty

    ~vkgv_gltf() {
        for (vkgv_mesh* m : meshes) vkgv_mesh_free(m);
    }
};

namespace {

// The asset version and the extensions it requires.
void check_asset(const JValue& root) {
    const JValue* asset = root.get("asset");
    if (!asset || !asset->get("version") || asset->get("version")->kind != JValue::String ||
        asset->get("version")->s.rfind("2.", 0) != 0)
        fail("not a glTF 2.0 asset");
    for (const JValue& e : array_of(root, "extensionsRequired").items) {
        if (e.kind != JValue::String) continue;
        // the extensions the reference enables in its parser (assets.cpp:536-541);
        // KHR_lights_punctual is read by nothing on this path
        static const char* const kKnown[] = {"EXT_meshopt_compression", "KHR_mesh_quantization",
                                             "KHR_texture_transform", "KHR_texture_basisu", "MSFT_texture_dds",
                                             "KHR_lights_punctual"};
        bool known = false;
        for (const char* k : kKnown) known = known || e.s == k;
        if (!known) fail("required extension " + e.s + " is not supported");
    }
}

// The encoded bytes of a glTF image: a base64 data URI, a file next to the
// asset, or a bufferView.
std::vector<uint8_t> image_bytes(const JValue& img, const JValue& root, const std::vector<std::vector<uint8_t>>& buffers,
                                 const std::string& dir) {
    if (const JValue* uri = img.get("uri")) {
        if (uri->kind != JValue::String) fail("image.uri must be a string");
        if (uri->s.rfind("data:", 0) == 0) {
            const size_t comma = uri->s.find(',');
            if (comma == std::string::npos || uri->s.find(";base64") == std::string::npos)
                fail("only base64 data URIs are supported");
            return base64(uri->s, comma + 1);
        }
        return read_file(dir + percent_decode(uri->s));
    }
    const int64_t bv = index_of(img, "bufferView");
    const JValue& views = array_of(root, "bufferViews");
    if (bv < 0 || size_t(bv) >= views.items.size()) fail("image without uri or a valid bufferView");
    const JValue& v = views.items[size_t(bv)];
    const int64_t b = index_of(v, "buffer"), off = index_of(v, "byteOffset", 0), len = index_of(v, "byteLength");
    if (b < 0 || size_t(b) >= buffers.size() || len < 0 || size_t(off + len) > buffers[size_t(b)].size())
        fail("image bufferView out of range");
    const uint8_t* base = buffers[size_t(b)].data() + off;
    return std::vector<uint8_t>(base, base + len);
}

void import_asset(vkgv_gltf& G, const JValue& root, const std::vector<std::vector<uint8_t>>& buffers,
                  const std::vector<bool>& placeholder, uint32_t flags, const std::string& dir) {
    Reader R(root, buffers, placeholder);

    // primitives (assets.cpp:288-430): positions, indices (generated when
    // absent), meshlets of 64 vertices / 124 triangles; colour and UV are
    // kept when present (the textured resolve reads them)
    const JValue& meshes = array_of(root, "meshes");
    G.mesh_offsets.assign(1, 0);
    for (size_t mi = 0; mi < meshes.items.size(); ++mi) {
        for (const JValue& p : array_of(meshes.items[mi], "primitives").items) {
            const int64_t mode = index_of(p, "mode", 4);
            if (mode != 4) fail("only TRIANGLES primitives are supported (mode " + std::to_string(mode) + ")");
            const JValue* attrs = p.get("attributes");
            if (!attrs || !attrs->get("POSITION")) fail("primitive without POSITION");
            const Accessor& pa = R.accessor(index_of(*attrs, "POSITION"));
            if (pa.ncomp != 3) fail("POSITION must be VEC3");
            std::vector<float> pos = R.floats(pa);
            if (pa.count == 0) fail("primitive with no vertices");
            std::vector<uint32_t> idx;
            const int64_t ia = index_of(p, "indices");
            if (ia >= 0) {
                idx = R.indices(R.accessor(ia));
            } else {
                idx.resize(pa.count);
                for (size_t k = 0; k < pa.count; ++k) idx[k] = uint32_t(k);
            }
            if (idx.size() % 3) fail("triangle list index count is not a multiple of 3");
            for (uint32_t v : idx)
                if (v >= pa.count) fail("index out of range");
            vkgv_mesh* m = vkgv_mesh_from_arrays(pos.data(), uint32_t(pa.count), idx.data(), uint32_t(idx.size() / 3));
            if (!m) fail("mesh construction failed");
            G.meshes.push_back(m);
            std::vector<float> rgba, uv;
            if (attrs->get("COLOR_0")) {
                const Accessor& ca = R.accessor(index_of(*attrs, "COLOR_0"));
                if (ca.count != pa.count || (ca.ncomp != 3 && ca.ncomp != 4)) fail("COLOR_0 must be VEC3 or VEC4");
                std::vector<float> c = R.floats(ca);
                rgba.assign(pa.count * 4, 1.0f);
                for (size_t k = 0; k < pa.count; ++k)
                    for (uint32_t j = 0; j < ca.ncomp; ++j) rgba[4 * k + j] = c[k * ca.ncomp + j];
            }
            if (attrs->get("TEXCOORD_0")) {
                const Accessor& ta = R.accessor(index_of(*attrs, "TEXCOORD_0"));
                if (ta.count != pa.count || ta.ncomp != 2) fail("TEXCOORD_0 must be VEC2");
                uv = R.floats(ta);
            }
            if (!rgba.empty() || !uv.empty())
                vkgv_mesh_set_attributes(m, rgba.empty() ? nullptr : rgba.data(), uv.empty() ? nullptr : uv.data());
            if (vkgv_mesh_build_meshlets(m, VKGV_MAX_VERTICES, VKGV_BUILDER_MAX_TRIANGLES) != VKGV_OK)
                fail("meshlet build failed");
            vkgv_mesh_info info;
            vkgv_mesh_get_info(m, &info);
            G.meshlet_counts.push_back(info.meshlet_count);
            const int64_t mat = index_of(p, "material");
            G.prim_material.push_back(mat >= 0 ? uint32_t(mat + 1) : 0u);  // assets.cpp:290-293
            G.prim_mesh.push_back(uint32_t(mi));
            G.mesh_primitives.push_back(uint32_t(G.meshes.size() - 1));
        }
        G.mesh_offsets.push_back(uint32_t(G.mesh_primitives.size()));
    }

    // materials (assets.cpp:474-518): index 0 is the glTF default material
    const JValue& mats = array_of(root, "materials");
    G.materials.assign(mats.items.size() + 1, vkgv_material{});
    for (vkgv_material& m : G.materials) {
        for (int k = 0; k < 4; ++k) m.albedo_factor[k] = 1.0f;
        m.albedo_index = VKGV_INVALID_HANDLE;
        m.uv_scale[0] = m.uv_scale[1] = 1.0f;
        m.alpha_cutoff = 0.5f;
    }
    for (size_t i = 0; i < mats.items.size(); ++i) {
        const JValue& jm = mats.items[i];
        vkgv_material& m = G.materials[i + 1];
        if (const JValue* pbr = jm.get("pbrMetallicRoughness")) {
            if (const JValue* f = pbr->get("baseColorFactor")) {
                if (f->kind != JValue::Array || f->items.size() != 4) fail("baseColorFactor must have 4 numbers");
                for (int k = 0; k < 4; ++k) m.albedo_factor[k] = float(f->items[k].n);
            }
            const JValue* tex = pbr->get("baseColorTexture");
            if (tex && (flags & VKGV_GLTF_TEXTURE_REFERENCES)) {
                m.albedo_index = uint32_t(index_of(*tex, "index"));
                const JValue* ext = tex->get("extensions");
                const JValue* tt = ext ? ext->get("KHR_texture_transform") : nullptr;
                if (tt) {
                    if (const JValue* o = tt->get("offset"))
                        for (int k = 0; k < 2 && k < int(o->items.size()); ++k) m.uv_offset[k] = float(o->items[k].n);
                    if (const JValue* s = tt->get("scale"))
                        for (int k = 0; k < 2 && k < int(s->items.size()); ++k) m.uv_scale[k] = float(s->items[k].n);
                    m.uv_rotation = float(num(*tt, "rotation", 0.0));
                }
            }
        }
        m.alpha_cutoff = float(num(jm, "alphaCutoff", 0.5));
        const JValue* ds = jm.get("doubleSided");
        m.double_sided = (ds && ds->kind == JValue::Bool && ds->b) ? 1u : 0u;
    }
    G.texture_count = uint32_t(array_of(root, "textures").items.size());
    G.image_count = uint32_t(array_of(root, "images").items.size());
    if (flags & VKGV_GLTF_IMAGES) {
        // each texture's image: a MSFT_texture_dds source takes precedence;
        // a KHR_texture_basisu (KTX2) source is used only without a base
        // source, which then is the fallback for BasisU-compressed KTX2
        const JValue& images = array_of(root, "images");
        const JValue& textures = array_of(root, "textures");
        G.texture_images.assign(textures.items.size(), std::vector<uint8_t>());
        for (size_t t = 0; t < textures.items.size(); ++t) {
            const JValue& tx = textures.items[t];
            int64_t src = index_of(tx, "source");
            if (const JValue* ext = tx.get("extensions")) {
                if (const JValue* ktx = ext->get("KHR_texture_basisu"))
                    if (src < 0) src = index_of(*ktx, "source");
                if (const JValue* dds = ext->get("MSFT_texture_dds")) src = index_of(*dds, "source", src);
            }
            if (src < 0) continue;
            if (size_t(src) >= images.items.size()) fail("texture source out of range");
            G.texture_images[t] = image_bytes(images.items[size_t(src)], root, buffers, dir);
        }
    }

    // nodes (DecomposeNodeMatrices) and the first scene's roots
    // (world.cpp:55-76: scenes.front().nodeIndices)
    const JValue& nodes = array_of(root, "nodes");
    const size_t N = nodes.items.size();
    G.nodes.assign(N, vkgv_node{});
    for (size_t n = 0; n < N; ++n) {
        const JValue& jn = nodes.items[n];
        vkgv_node& nd = G.nodes[n];
        nd.rotation[3] = 1.0f;
        nd.scale[0] = nd.scale[1] = nd.scale[2] = 1.0f;
        if (const JValue* mtx = jn.get("matrix")) {
            if (mtx->kind != JValue::Array || mtx->items.size() != 16) fail("node.matrix must have 16 numbers");
            double m[16];
            for (int k = 0; k < 16; ++k) m[k] = mtx->items[k].n;
            decompose(m, nd.translation, nd.rotation, nd.scale);
        } else {
            if (const JValue* t = jn.get("translation"))
                for (int k = 0; k < 3 && k < int(t->items.size()); ++k) nd.translation[k] = float(t->items[k].n);
            if (const JValue* r = jn.get("rotation"))
                for (int k = 0; k < 4 && k < int(r->items.size()); ++k) nd.rotation[k] = float(r->items[k].n);
            if (const JValue* s = jn.get("scale"))
                for (int k = 0; k < 3 && k < int(s->items.size()); ++k) nd.scale[k] = float(s->items[k].n);
        }
        const int64_t mesh = index_of(jn, "mesh");
        if (mesh >= int64_t(meshes.items.size())) fail("node.mesh out of range");
        nd.mesh_index = mesh >= 0 ? uint32_t(mesh) : VKGV_INVALID_HANDLE;
        nd.first_child = uint32_t(G.children.size());
        for (const JValue& c : array_of(jn, "children").items) {
            if (!c.is_num() || c.n < 0 || size_t(c.n) >= N) fail("node child out of range");
            G.children.push_back(uint32_t(c.n));
        }
        nd.child_count = uint32_t(G.children.size()) - nd.first_child;
    }
    const JValue& scenes = array_of(root, "scenes");
    if (!scenes.items.empty())
        for (const JValue& r : array_of(scenes.items[0], "nodes").items) {
            if (!r.is_num() || r.n < 0 || size_t(r.n) >= N) fail("scene node out of range");
            G.roots.push_back(uint32_t(r.n));
        }

    // animations (assets.hpp:37-47; channels in animation, channel order)
    for (const JValue& an : array_of(root, "animations").items) {
        const uint32_t base = uint32_t(G.samplers.size());
        const JValue& samps = array_of(an, "samplers");
        for (const JValue& s : samps.items) {
            const Accessor& in = R.accessor(index_of(s, "input"));
            const Accessor& out = R.accessor(index_of(s, "output"));
            if (in.ncomp != 1 || in.count == 0) fail("animation input must be a non-empty SCALAR accessor");
            uint32_t interp = VKGV_INTERP_LINEAR;
            if (const JValue* i = s.get("interpolation")) {
                if (i->s == "STEP") interp = VKGV_INTERP_STEP;
                else if (i->s == "CUBICSPLINE") interp = VKGV_INTERP_CUBICSPLINE;
                else if (i->s != "LINEAR") fail("unknown interpolation " + i->s);
            }
            std::vector<float> k = R.floats(in);
            std::vector<float> v = R.floats(out);
            vkgv_anim_sampler as{};
            as.input_count = uint32_t(in.count);
            as.output_count = uint32_t(out.count);
            as.interpolation = interp;
            as.components = out.ncomp;
            k.insert(k.end(), v.begin(), v.end());
            G.keys.push_back(std::move(k));
            G.samplers.push_back(as);
        }
        for (const JValue& ch : array_of(an, "channels").items) {
            vkgv_anim_channel c{};
            const int64_t s = index_of(ch, "sampler");
            if (s < 0 || size_t(s) >= samps.items.size()) fail("channel sampler out of range");
            c.sampler = base + uint32_t(s);
            const JValue* target = ch.get("target");
            if (!target) fail("channel without target");
            const int64_t node = index_of(*target, "node");
            c.node = node >= 0 ? uint32_t(node) : VKGV_INVALID_HANDLE;
            const JValue* path = target->get("path");
            if (!path || path->kind != JValue::String) fail("channel target without path");
            if (path->s == "translation") c.path = VKGV_PATH_TRANSLATION;
            else if (path->s == "rotation") c.path = VKGV_PATH_ROTATION;
            else if (path->s == "scale") c.path = VKGV_PATH_SCALE;
            else if (path->s == "weights") c.path = VKGV_PATH_WEIGHTS;
            else fail("unknown channel path " + path->s);
            G.channels.push_back(c);
        }
    }
    for (size_t i = 0; i < G.samplers.size(); ++i) {
        G.samplers[i].input = G.keys[i].data();
        G.samplers[i].output = G.keys[i].data() + G.samplers[i].input_count;
    }
}

void put_error(char* error, uint32_t cap, const std::string& m) {
    if (!error || !cap) return;
    std::snprintf(error, cap, "%s", m.c_str());
}

}  // namespace

extern "C" int vkgv_gltf_load(const char* path, uint32_t flags, vkgv_gltf** out, char* error, uint32_t error_capacity) {
    if (!path || !out) return VKGV_INVALID_ARG;
    *out = nullptr;
    vkgv_gltf* G = new (std::nothrow) vkgv_gltf();
    if (!G) return VKGV_OUT_OF_MEMORY;
    try {
        std::vector<uint8_t> file = read_file(path);
        std::string dir(path);
        const size_t slash = dir.find_last_of('/');
        dir = slash == std::string::npos ? std::string() : dir.substr(0, slash + 1);
        const char* json = reinterpret_cast<const char*>(file.data());
        size_t json_len = file.size();
        std::vector<uint8_t> glb_bin;
        bool have_bin = false;
        uint32_t magic = 0;
        if (file.size() >= 4) std::memcpy(&magic, file.data(), 4);
        if (magic == 0x46546C67u) {  // "glTF": the binary container
            uint32_t hdr[3];
            if (file.size() < 20) fail("truncated GLB header");
            std::memcpy(hdr, file.data(), 12);
            if (hdr[1] != 2) fail("GLB version must be 2");
            if (hdr[2] > file.size()) fail("GLB length exceeds the file");
            size_t at = 12;
            bool have_json = false;
            while (at + 8 <= hdr[2]) {
                uint32_t len, type;
                std::memcpy(&len, file.data() + at, 4);
                std::memcpy(&type, file.data() + at + 4, 4);
                if (at + 8 + size_t(len) > hdr[2]) fail("GLB chunk exceeds the file");
                if (type == 0x4E4F534Au && !have_json) {
                    json = reinterpret_cast<const char*>(file.data() + at + 8);
                    json_len = len;
                    have_json = true;
                } else if (type == 0x004E4942u && !have_bin) {
                    glb_bin.assign(file.data() + at + 8, file.data() + at + 8 + len);
                    have_bin = true;
                }
                at += 8 + size_t(len);
            }
            if (!have_json) fail("GLB without a JSON chunk");
        }
        JValue root;
        std::string err;
        if (!JsonParser(json, json_len).parse(root, err)) fail(err);
        if (root.kind != JValue::Object) fail("the glTF root must be an object");
        check_asset(root);
        std::vector<std::vector<uint8_t>> buffers;
        const JValue& bufs = array_of(root, "buffers");
        std::vector<bool> placeholder(bufs.items.size(), false);
        for (size_t i = 0; i < bufs.items.size(); ++i) {
            const JValue& b = bufs.items[i];
            const int64_t blen = index_of(b, "byteLength");
            if (blen < 0) fail("buffer.byteLength missing");
            const size_t length = size_t(blen);
            const JValue* uri = b.get("uri");
            // EXT_meshopt_compression's fallback buffer holds the uncompressed
            // data for loaders without the extension: never read
            const JValue* bext = b.get("extensions");
            const JValue* mc = bext ? bext->get("EXT_meshopt_compression") : nullptr;
            const JValue* fb = mc ? mc->get("fallback") : nullptr;
            if (fb && fb->kind == JValue::Bool && fb->b && !(i == 0 && !uri && have_bin)) {
                placeholder[i] = true;
                buffers.emplace_back();
                continue;
            }
            std::vector<uint8_t> data;
            if (!uri) {
                if (i != 0 || !have_bin) fail("buffer without uri outside a GLB");
                data = glb_bin;
            } else if (uri->s.rfind("data:", 0) == 0) {
                const size_t comma = uri->s.find(',');
                if (comma == std::string::npos || uri->s.find(";base64") == std::string::npos)
                    fail("only base64 data URIs are supported");
                data = base64(uri->s, comma + 1);
            } else {
                data = read_file(dir + percent_decode(uri->s));
            }
            if (data.size() < length) fail("buffer shorter than its byteLength");
            data.resize(length);
            buffers.push_back(std::move(data));
        }
        import_asset(*G, root, buffers, placeholder, flags, dir);
    } catch (const ImportError& e) {
        put_error(error, error_capacity, e.msg);
        delete G;
        return VKGV_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        put_error(error, error_capacity, "out of host memory");
        delete G;
        return VKGV_OUT_OF_MEMORY;
    }
    *out = G;
    return VKGV_OK;
}

extern "C" int vkgv_gltf_get_info(const vkgv_gltf* g, vkgv_gltf_info* out) {
    if (!g || !out) return VKGV_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->primitive_count = uint32_t(g->meshes.size());
    out->material_count = uint32_t(g->materials.size());
    out->mesh_count = uint32_t(g->mesh_offsets.size() - 1);
    out->node_count = uint32_t(g->nodes.size());
    out->root_count = uint32_t(g->roots.size());
    out->sampler_count = uint32_t(g->samplers.size());
    out->channel_count = uint32_t(g->channels.size());
    out->texture_count = g->texture_count;
    out->image_count = g->image_count;
    return VKGV_OK;
}

extern "C" int vkgv_gltf_get_primitive(const vkgv_gltf* g, uint32_t index, vkgv_gltf_primitive* out) {
    if (!g || !out || index >= g->meshes.size()) return VKGV_INVALID_ARG;
    out->mesh = g->meshes[index];
    out->material_index = g->prim_material[index];
    out->mesh_index = g->prim_mesh[index];
    out->meshlet_count = g->meshlet_counts[index];
    return VKGV_OK;
}

extern "C" int vkgv_gltf_get_materials(const vkgv_gltf* g, vkgv_material* out, uint32_t capacity) {
    if (!g || (!out && capacity)) return VKGV_INVALID_ARG;
    if (capacity < g->materials.size()) return VKGV_LIMIT_EXCEEDED;
    std::memcpy(out, g->materials.data(), sizeof(vkgv_material) * g->materials.size());
    return VKGV_OK;
}

extern "C" int vkgv_gltf_get_world(const vkgv_gltf* g, vkgv_world_desc* out) {
    if (!g || !out) return VKGV_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    out->nodes = g->nodes.data();
    out->node_count = uint32_t(g->nodes.size());
    out->children = g->children.data();
    out->child_count = uint32_t(g->children.size());
    out->roots = g->roots.data();
    out->root_count = uint32_t(g->roots.size());
    out->mesh_count = uint32_t(g->mesh_offsets.size() - 1);
    out->mesh_offsets = g->mesh_offsets.data();
    out->mesh_primitives = g->mesh_primitives.data();
    out->primitive_meshlet_counts = g->meshlet_counts.data();
    out->primitive_count = uint32_t(g->meshlet_counts.size());
    out->samplers = g->samplers.data();
    out->sampler_count = uint32_t(g->samplers.size());
    out->channels = g->channels.data();
    out->channel_count = uint32_t(g->channels.size());
    return VKGV_OK;
}

extern "C" int vkgv_gltf_get_texture_image(const vkgv_gltf* g, uint32_t texture, vkgv_gltf_image* out) {
    if (!g || !out) return VKGV_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    if (texture >= g->texture_images.size()) return VKGV_INVALID_ARG;
    const std::vector<uint8_t>& d = g->texture_images[texture];
    out->data = d.empty() ? nullptr : d.data();
    out->size = d.size();
    static const uint8_t png[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    static const uint8_t ktx2[8] = {0xAB, 0x4B, 0x54, 0x58, 0x20, 0x32, 0x30, 0xBB};
    if (d.size() >= 8 && !std::memcmp(d.data(), png, 8)) out->kind = VKGV_IMAGE_PNG;
    else if (d.size() >= 4 && !std::memcmp(d.data(), "DDS ", 4)) out->kind = VKGV_IMAGE_DDS;
    else if (d.size() >= 3 && d[0] == 0xFF && d[1] == 0xD8 && d[2] == 0xFF) out->kind = VKGV_IMAGE_JPEG;
    else if (d.size() >= 8 && !std::memcmp(d.data(), ktx2, 8)) out->kind = VKGV_IMAGE_KTX2;
    else out->kind = VKGV_IMAGE_UNKNOWN;
    return VKGV_OK;
}

extern "C" void vkgv_gltf_free(vkgv_gltf* g) { delete g; }
