// console.cpp - headless RuntimeConsole -> SimParams mapping (see
// include/pbf/console.h) and its C ABI (pbf_console_*).
#include "../../include/pbf/console.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "../../include/pbf/pbf.h"
#include "handle.h"

namespace console {
namespace {

// ------------------------------------------------------------------ JSON
// A small JSON reader: objects (duplicate keys: the last one counts),
// arrays, numbers, strings (with escapes), true / false / null.
struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;

    const JValue* find(const char* key) const {
        if (kind != Object) return nullptr;
        for (auto it = obj.rbegin(); it != obj.rend(); ++it)
            if (it->first == key) return &it->second;
        return nullptr;
    }
};

class JsonReader {
public:
    explicit JsonReader(const std::string& t) : s_(t) {}

    bool parse(JValue& out, std::string& err) {
        skip();
        if (!value(out, 0)) {
            err = "config: json parse error at offset " + std::to_string(pos_) + ": " + why_;
            return false;
        }
        skip();
        if (pos_ != s_.size()) {
            err = "config: json parse error at offset " + std::to_string(pos_) + ": trailing characters";
            return false;
        }
        return true;
    }

private:
    static constexpr int kMaxDepth = 256;

    bool fail(const char* why) {
        why_ = why;
        return false;
    }
    void skip() {
        while (pos_ < s_.size() && (s_[pos_] == ' ' || s_[pos_] == '\t' || s_[pos_] == '\n' || s_[pos_] == '\r'))
            ++pos_;
    }
    bool literal(const char* word) {
        const size_t n = std::strlen(word);
        if (s_.compare(pos_, n, word) != 0) return fail("invalid literal");
        pos_ += n;
        return true;
    }
    bool value(JValue& v, int depth) {
        if (depth > kMaxDepth) return fail("nesting too deep");
        if (pos_ >= s_.size()) return fail("unexpected end");
        const char c = s_[pos_];
        if (c == '{') return object(v, depth);
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v.kind = JValue::String;
            return string(v.str);
        }
        if (c == 't') {
            v.kind = JValue::Bool;
            v.b = true;
            return literal("true");
        }
        if (c == 'f') {
            v.kind = JValue::Bool;
            v.b = false;
            return literal("false");
        }
        if (c == 'n') {
            v.kind = JValue::Null;
            return literal("null");
        }
        return number(v);
    }
    bool object(JValue& v, int depth) {
        v.kind = JValue::Object;
        ++pos_;
        skip();
        if (pos_ < s_.size() && s_[pos_] == '}') {
            ++pos_;
            return true;
        }
        for (;;) {
            skip();
            if (pos_ >= s_.size() || s_[pos_] != '"') return fail("expected a key");
            std::string key;
            if (!string(key)) return false;
            skip();
            if (pos_ >= s_.size() || s_[pos_] != ':') return fail("expected ':'");
            ++pos_;
            skip();
            JValue item;
            if (!value(item, depth + 1)) return false;
            v.obj.emplace_back(std::move(key), std::move(item));
            skip();
            if (pos_ < s_.size() && s_[pos_] == ',') {
                ++pos_;
                continue;
            }
            if (pos_ < s_.size() && s_[pos_] == '}') {
                ++pos_;
                return true;
            }
            return fail("expected ',' or '}'");
        }
    }
    bool array(JValue& v, int depth) {
        v.kind = JValue::Array;
        ++pos_;
        skip();
        if (pos_ < s_.size() && s_[pos_] == ']') {
            ++pos_;
            return true;
        }
        for (;;) {
            skip();
            JValue item;
            if (!value(item, depth + 1)) return false;
            v.arr.push_back(std::move(item));
            skip();
            if (pos_ < s_.size() && s_[pos_] == ',') {
                ++pos_;
                continue;
            }
            if (pos_ < s_.size() && s_[pos_] == ']') {
                ++pos_;
                return true;
            }
            return fail("expected ',' or ']'");
        }
    }
    static void put_utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) {
            out += char(cp);
        } else if (cp < 0x800) {
            out += char(0xC0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += char(0xE0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        } else {
            out += char(0xF0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3F));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        }
    }
    bool hex4(uint32_t& cp) {
        if (pos_ + 4 > s_.size()) return fail("short \\u escape");
        cp = 0;
        for (int i = 0; i < 4; ++i) {
            const char h = s_[pos_++];
            cp <<= 4;
            if (h >= '0' && h <= '9') cp |= uint32_t(h - '0');
            else if (h >= 'a' && h <= 'f') cp |= uint32_t(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') cp |= uint32_t(h - 'A' + 10);
            else return fail("bad \\u escape");
        }
        return true;
    }
    bool string(std::string& out) {
        ++pos_;  // opening quote
        while (pos_ < s_.size()) {
            const unsigned char c = static_cast<unsigned char>(s_[pos_++]);
            if (c == '"') return true;
            if (c < 0x20) return fail("control character in string");
            if (c != '\\') {
                out += char(c);
                continue;
            }
            if (pos_ >= s_.size()) return fail("unexpected end");
            const char e = s_[pos_++];
            switch (e) {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u': {
                uint32_t cp;
                if (!hex4(cp)) return false;
                if (cp >= 0xD800 && cp < 0xDC00 && pos_ + 1 < s_.size() && s_[pos_] == '\\' && s_[pos_ + 1] == 'u') {
                    pos_ += 2;
                    uint32_t lo;
                    if (!hex4(lo)) return false;
                    if (lo >= 0xDC00 && lo < 0xE000) cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                put_utf8(out, cp);
                break;
            }
            default: return fail("bad escape");
            }
        }
        return fail("unterminated string");
    }
    bool number(JValue& v) {
        const size_t b = pos_;
        if (pos_ < s_.size() && s_[pos_] == '-') ++pos_;
        if (pos_ >= s_.size() || !(s_[pos_] >= '0' && s_[pos_] <= '9')) return fail("invalid value");
        if (s_[pos_] == '0') {
            ++pos_;
        } else {
            while (pos_ < s_.size() && s_[pos_] >= '0' && s_[pos_] <= '9') ++pos_;
        }
        if (pos_ < s_.size() && s_[pos_] == '.') {
            ++pos_;
            if (pos_ >= s_.size() || !(s_[pos_] >= '0' && s_[pos_] <= '9')) return fail("invalid number");
            while (pos_ < s_.size() && s_[pos_] >= '0' && s_[pos_] <= '9') ++pos_;
        }
        if (pos_ < s_.size() && (s_[pos_] == 'e' || s_[pos_] == 'E')) {
            ++pos_;
            if (pos_ < s_.size() && (s_[pos_] == '+' || s_[pos_] == '-')) ++pos_;
            if (pos_ >= s_.size() || !(s_[pos_] >= '0' && s_[pos_] <= '9')) return fail("invalid number");
            while (pos_ < s_.size() && s_[pos_] >= '0' && s_[pos_] <= '9') ++pos_;
        }
        const std::string text = s_.substr(b, pos_ - b);
        v.kind = JValue::Number;
        v.num = std::strtod(text.c_str(), nullptr);
        return true;
    }

    const std::string& s_;
    size_t pos_ = 0;
    const char* why_ = "";
};

// Typed reads of the config's values, with the conversions of the
// reference's reader (nlohmann::json get<T>): numbers to float / int by
// conversion, booleans and strings only from their own type.
struct TypeError {};
float as_float(const JValue& v) {
    if (v.kind != JValue::Number) throw TypeError{};
    return float(v.num);
}
int as_int(const JValue& v) {
    if (v.kind != JValue::Number) throw TypeError{};
    const double d = std::trunc(v.num);
    return d >= double(INT_MAX) ? INT_MAX : d <= double(INT_MIN) ? INT_MIN : int(d);
}
bool as_bool(const JValue& v) {
    if (v.kind != JValue::Bool) throw TypeError{};
    return v.b;
}
const std::string& as_string(const JValue& v) {
    if (v.kind != JValue::String) throw TypeError{};
    return v.str;
}

// ------------------------------------------------------------- CubeMix
uint32_t clamp_u64_to_u32(uint64_t v) { return v > 0xFFFFFFFFull ? 0xFFFFFFFFu : uint32_t(v); }

uint32_t nearest_cube_root(uint64_t v) {
    if (v == 0) return 0;
    const long long r = std::llround(std::cbrt(double(v)));
    return uint32_t(std::max<long long>(1, r));
}

// Groups per layer, front-loaded: layer L gets remaining / (layers - L), at
// least one.
std::vector<uint32_t> layer_split(uint32_t groups, uint32_t layers, bool stopWhenDone) {
    std::vector<uint32_t> counts(layers, 0u);
    uint32_t remaining = groups;
    for (uint32_t L = 0; L < layers && (!stopWhenDone || remaining > 0); ++L) {
        uint32_t take = remaining / (layers - L);
        if (take == 0) take = 1;
        counts[L] = take;
        remaining -= take;
    }
    return counts;
}

float layer_height(const RuntimeConsole::Simulation& s, uint32_t layer, float h) {
    float y = s.cube_base_height + float(layer) * s.cube_layer_spacing_world;
    if (s.cube_layer_jitter_enable) {
        std::mt19937 rng(s.cube_layer_jitter_seed ^ layer);
        std::uniform_real_distribution<float> u(-1.f, 1.f);
        y += u(rng) * (s.cube_layer_jitter_scale_h * h);
    }
    return y;
}

void update_cube_mix(RuntimeConsole::Simulation& s) {
    using Sim = RuntimeConsole::Simulation;
    if (s.demoMode != Sim::DemoMode::CubeMix) return;
    s.cube_group_count = std::max(1u, std::min(s.cube_group_count, Sim::cube_group_count_max));
    if (s.cube_auto_partition) {
        // largest cubes of equal edge L whose G copies fit the requested count
        const uint64_t target = std::max(1u, s.numParticles);
        uint32_t L = nearest_cube_root(target);
        if (L == 0) L = 1;
        uint64_t per = uint64_t(L) * L * L;
        uint32_t G = uint32_t(std::max<uint64_t>(1ull, target / per));
        while (uint64_t(G) * L * L * L > target && L > 1) --L;
        while (uint64_t(G) * (L + 1) * (L + 1) * (L + 1) <= target) ++L;
        per = uint64_t(L) * L * L;
        while (uint64_t(G + 1) * per <= target && G + 1 <= Sim::cube_group_count_max) ++G;
        s.cube_edge_particles = L;
        s.cube_group_count = std::min(G, Sim::cube_group_count_max);
    }
    s.cube_particles_per_group =
        clamp_u64_to_u32(uint64_t(s.cube_edge_particles) * s.cube_edge_particles * s.cube_edge_particles);
    s.numParticles = s.cube_group_count * s.cube_particles_per_group;  // modulo 2^32, as the reference
    if (s.cube_layers < 1) s.cube_layers = 1;
    if (s.cube_layers > s.cube_group_count) s.cube_layers = s.cube_group_count;

    const std::vector<uint32_t> perLayer = layer_split(s.cube_group_count, s.cube_layers, true);
    const float h = (s.smoothingRadius > 1e-6f) ? s.smoothingRadius : 1e-6f;
    const float spacing = h * s.cube_lattice_spacing_factor_h;
    const float halfSide = (spacing * float(s.cube_edge_particles)) * 0.5f;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    uint32_t placed = 0;
    for (uint32_t layer = 0; layer < s.cube_layers && placed < s.cube_group_count; ++layer) {
        const uint32_t n = perLayer[layer];
        if (n == 0) continue;
        const uint32_t nx = uint32_t(std::ceil(std::sqrt(double(n))));
        const float y = layer_height(s, layer, h);
        for (uint32_t k = 0; k < n && placed < s.cube_group_count; ++k, ++placed) {
            const float c[3] = {float(k % nx) * s.cube_group_spacing_world, y,
                                float(k / nx) * s.cube_group_spacing_world};
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], c[a] - halfSide);
                hi[a] = std::max(hi[a], c[a] + halfSide);
            }
        }
    }
    if (lo[0] > hi[0] || lo[1] > hi[1] || lo[2] > hi[2]) {
        for (int a = 0; a < 3; ++a) {
            lo[a] = -halfSide;
            hi[a] = halfSide;
        }
    }
    if (s.cube_auto_fit_domain) {
        // the groups' box, its floor lowered to y = 0 or one half cube below
        // them, widened about its centre by the margin; the domain's floor
        // stays at y >= 0
        const float size[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
        const float mn[3] = {lo[0], std::min(0.f, lo[1] - halfSide), lo[2]};
        const float mx[3] = {lo[0] + size[0], lo[1] + size[1], lo[2] + size[2]};
        const float scale = (s.cube_domain_margin_scale < 1.0f) ? 1.0f : s.cube_domain_margin_scale;
        float centre[3], half[3];
        for (int a = 0; a < 3; ++a) {
            centre[a] = (mn[a] + mx[a]) * 0.5f;
            half[a] = (mx[a] - mn[a]) * 0.5f * scale;
        }
        s.gridMins = make_float3(centre[0] - half[0], std::max(0.f, centre[1] - half[1]), centre[2] - half[2]);
        s.gridMaxs = make_float3(centre[0] + half[0], centre[1] + half[1], centre[2] + half[2]);
    }
}

}  // namespace

RuntimeConsole::Simulation::Simulation() { refreshCubeMixDerived(); }

void RuntimeConsole::Simulation::refreshCubeMixDerived() { update_cube_mix(*this); }

void PrepareCubeMix(RuntimeConsole& c) { update_cube_mix(c.sim); }

void GenerateCubeMixCenters(const RuntimeConsole& c, std::vector<float3>& out) {
    out.clear();
    const auto& s = c.sim;
    if (s.demoMode != RuntimeConsole::Simulation::DemoMode::CubeMix) return;
    const std::vector<uint32_t> perLayer = layer_split(s.cube_group_count, s.cube_layers, false);
    const float h = (1e-6f > s.smoothingRadius) ? 1e-6f : s.smoothingRadius;
    out.reserve(s.cube_group_count);
    uint32_t placed = 0;
    for (uint32_t layer = 0; layer < s.cube_layers && placed < s.cube_group_count; ++layer) {
        const uint32_t n = perLayer[layer];
        const uint32_t nx = uint32_t(std::ceil(std::sqrt(double(n))));
        const float y = layer_height(s, layer, h);
        for (uint32_t k = 0; k < n && placed < s.cube_group_count; ++k, ++placed)
            out.push_back(make_float3(float(k % nx) * s.cube_group_spacing_world, y,
                                      float(k / nx) * s.cube_group_spacing_world));
    }
}

void BuildSimParams(const RuntimeConsole& c, sim::SimParams& out) {
    const auto& s = c.sim;
    out.numParticles = s.numParticles;
    out.maxParticles = s.maxParticles;
    out.dt = s.dt;
    out.cfl = s.cfl;
    out.gravity = s.gravity;
    out.restDensity = s.restDensity;
    out.solverIters = s.solverIters;
    out.maxNeighbors = (c.perf.neighbor_cap > 0) ? c.perf.neighbor_cap : s.maxNeighbors;
    out.boundaryRestitution = s.boundaryRestitution;
    out.pbf = s.pbf;
    out.xsph_c = s.xsph_c;
    // the console's stability switches override the tuning block
    out.pbf.xpbd_enable = s.xpbd_enable ? 1 : 0;
    out.pbf.compliance = s.xpbd_enable ? s.xpbd_compliance : 0.0f;
    out.pbf.lambda_warm_start_enable = s.lambda_warm_start_enable ? 1 : 0;
    out.pbf.lambda_warm_start_decay = s.lambda_warm_start_decay;
    out.pbf.semi_implicit_integration_enable = s.integrate_semi_implicit ? 1 : 0;

    // smoothing length: the kernel radius, or h_over_r particle radii
    const float rSafe = (1e-8f > s.particleRadiusWorld) ? 1e-8f : s.particleRadiusWorld;
    float h = (s.smoothingRadius > 0.f) ? s.smoothingRadius : 0.02f;
    if (s.deriveHFromRadius) {
        const float fromR = s.h_over_r * rSafe;
        if (fromR > 0.0f) h = fromR;
    }
    out.kernel = sim::MakeKernelCoeffs(h);

    float mass = s.particleMass;
    if (s.massMode == RuntimeConsole::Simulation::MassMode::UniformLattice) {
        const float spacing = ((s.lattice_spacing_factor_h > 0.f) ? s.lattice_spacing_factor_h : 1.0f) * h;
        mass = s.restDensity * spacing * spacing * spacing;
    } else if (s.massMode == RuntimeConsole::Simulation::MassMode::SphereByRadius) {
        const float pi = 3.14159265358979323846f;
        mass = s.particleVolumeScale * (4.0f / 3.0f) * pi * rSafe * rSafe * rSafe * s.restDensity;
    }
    out.particleMass = mass;

    float cell = s.cellSize;
    if (cell <= 0.0f) {
        const float m = (c.perf.grid_cell_size_multiplier > 0.0f) ? c.perf.grid_cell_size_multiplier : 1.0f;
        cell = (1e-6f > m * h) ? 1e-6f : m * h;
    }
    out.grid.mins = s.gridMins;
    out.grid.maxs = s.gridMaxs;
    out.grid.cellSize = cell;
    const float ext[3] = {s.gridMaxs.x - s.gridMins.x, s.gridMaxs.y - s.gridMins.y, s.gridMaxs.z - s.gridMins.z};
    int d[3];
    for (int a = 0; a < 3; ++a) d[a] = std::max(1, int(std::ceil(ext[a] / cell)));
    out.grid.dim = make_int3(d[0], d[1], d[2]);
}

void BuildDeviceParams(const RuntimeConsole& c, sim::DeviceParams& out) {
    sim::SimParams sp{};
    BuildSimParams(c, sp);
    out = sim::MakeDeviceParams(sp);
}

void SanitizeSimParams(const RuntimeConsole& c, sim::SimParams& sp) {
    sp.solverIters = std::min(64, std::max(1, sp.solverIters));
    if (sp.maxNeighbors < 8) sp.maxNeighbors = 8;
    if (c.perf.neighbor_cap > 0 && sp.maxNeighbors > c.perf.neighbor_cap) sp.maxNeighbors = c.perf.neighbor_cap;
    if (sp.maxNeighbors > 1024) sp.maxNeighbors = 1024;
    if (sp.sortEveryN < 1) sp.sortEveryN = 1;
}

bool MergeConfigJson(RuntimeConsole& c, const std::string& text, std::string* activeProfile, std::string* err) {
    JValue j;
    std::string e;
    if (!JsonReader(text).parse(j, e)) {
        if (err) *err = e;
        return false;
    }
    RuntimeConsole m = c;  // merged into a copy: all keys or none
    std::string profile = activeProfile ? *activeProfile : std::string();
    try {
        if (const JValue* p = j.find("performance"); p && p->kind == JValue::Object) {
            if (const JValue* v = p->find("grid_cell_size_multiplier")) m.perf.grid_cell_size_multiplier = as_float(*v);
            if (const JValue* v = p->find("neighbor_cap")) m.perf.neighbor_cap = as_int(*v);
            if (const JValue* v = p->find("launch_bounds_tbs")) m.perf.launch_bounds_tbs = as_int(*v);
            if (const JValue* v = p->find("min_blocks_per_sm")) m.perf.min_blocks_per_sm = as_int(*v);
            if (const JValue* v = p->find("use_hashed_grid")) m.perf.use_hashed_grid = as_bool(*v);
            if (const JValue* v = p->find("sort_compact_every_n")) m.perf.sort_compact_every_n = as_int(*v);
            if (const JValue* v = p->find("compact_binary_search")) m.perf.compact_binary_search = as_bool(*v);
            if (const JValue* v = p->find("log_grid_compact_stats")) m.perf.log_grid_compact_stats = as_bool(*v);
        }
        if (const JValue* s = j.find("simulation"); s && s->kind == JValue::Object) {
            if (const JValue* v = s->find("cfl")) m.sim.cfl = as_float(*v);
            if (const JValue* v = s->find("rest_density")) m.sim.restDensity = as_float(*v);
            if (const JValue* v = s->find("kernel_radius")) m.sim.smoothingRadius = as_float(*v);
            if (const JValue* v = s->find("solver_iterations")) m.sim.solverIters = as_int(*v);
            if (const JValue* v = s->find("max_neighbors")) m.sim.maxNeighbors = as_int(*v);
            if (const JValue* v = s->find("xsph_c")) m.sim.xsph_c = as_float(*v);
        }
        if (const JValue* p = j.find("profile"); p && p->kind == JValue::String) profile = as_string(*p);
        const JValue* profiles = j.find("profiles");
        if (!profile.empty() && profiles && profiles->kind == JValue::Object) {
            if (const JValue* P = profiles->find(profile.c_str()); P && P->kind == JValue::Object) {
                if (const JValue* ps = P->find("simulation"); ps && ps->kind == JValue::Object) {
                    if (const JValue* v = ps->find("solver_iterations")) m.sim.solverIters = as_int(*v);
                    if (const JValue* v = ps->find("max_neighbors")) m.sim.maxNeighbors = as_int(*v);
                }
                if (const JValue* pp = P->find("performance"); pp && pp->kind == JValue::Object) {
                    if (const JValue* v = pp->find("neighbor_cap")) m.perf.neighbor_cap = as_int(*v);
                }
            }
        }
    } catch (const TypeError&) {
        if (err) *err = "config: json type error: a known key has a value of the wrong type";
        return false;
    }
    PrepareCubeMix(m);
    c = m;
    if (activeProfile) *activeProfile = profile;
    return true;
}

}  // namespace console

// ------------------------------------------------------------------ C ABI
struct pbf_console {
    console::RuntimeConsole c;
    std::string profile;
};

namespace {

using Sim = console::RuntimeConsole::Simulation;

enum class FieldType { F32, I32, U32, Bool, MassMode };
struct Field {
    const char* name;
    FieldType type;
    void* (*at)(console::RuntimeConsole&);
};

#define PBF_SIM_FIELD(nm, member, ty) \
    {"sim." nm, FieldType::ty, [](console::RuntimeConsole& c) -> void* { return &c.sim.member; }}
#define PBF_PERF_FIELD(nm, member, ty) \
    {"perf." nm, FieldType::ty, [](console::RuntimeConsole& c) -> void* { return &c.perf.member; }}
#define PBF_TUNING_FIELD(nm, ty) \
    {"sim.pbf." #nm, FieldType::ty, [](console::RuntimeConsole& c) -> void* { return &c.sim.pbf.nm; }}

const Field kFields[] = {
    PBF_SIM_FIELD("numParticles", numParticles, U32),
    PBF_SIM_FIELD("maxParticles", maxParticles, U32),
    PBF_SIM_FIELD("dt", dt, F32),
    PBF_SIM_FIELD("cfl", cfl, F32),
    PBF_SIM_FIELD("gravity.x", gravity.x, F32),
    PBF_SIM_FIELD("gravity.y", gravity.y, F32),
    PBF_SIM_FIELD("gravity.z", gravity.z, F32),
    PBF_SIM_FIELD("restDensity", restDensity, F32),
    PBF_SIM_FIELD("massMode", massMode, MassMode),
    PBF_SIM_FIELD("lattice_spacing_factor_h", lattice_spacing_factor_h, F32),
    PBF_SIM_FIELD("particleMass", particleMass, F32),
    PBF_SIM_FIELD("particleVolumeScale", particleVolumeScale, F32),
    PBF_SIM_FIELD("particleRadiusWorld", particleRadiusWorld, F32),
    PBF_SIM_FIELD("deriveHFromRadius", deriveHFromRadius, Bool),
    PBF_SIM_FIELD("h_over_r", h_over_r, F32),
    PBF_SIM_FIELD("xsph_c", xsph_c, F32),
    PBF_SIM_FIELD("smoothingRadius", smoothingRadius, F32),
    PBF_SIM_FIELD("gridMins.x", gridMins.x, F32),
    PBF_SIM_FIELD("gridMins.y", gridMins.y, F32),
    PBF_SIM_FIELD("gridMins.z", gridMins.z, F32),
    PBF_SIM_FIELD("gridMaxs.x", gridMaxs.x, F32),
    PBF_SIM_FIELD("gridMaxs.y", gridMaxs.y, F32),
    PBF_SIM_FIELD("gridMaxs.z", gridMaxs.z, F32),
    PBF_SIM_FIELD("cellSize", cellSize, F32),
    PBF_SIM_FIELD("solverIters", solverIters, I32),
    PBF_SIM_FIELD("maxNeighbors", maxNeighbors, I32),
    PBF_SIM_FIELD("boundaryRestitution", boundaryRestitution, F32),
    PBF_SIM_FIELD("cube_auto_partition", cube_auto_partition, Bool),
    PBF_SIM_FIELD("cube_group_count", cube_group_count, U32),
    PBF_SIM_FIELD("cube_edge_particles", cube_edge_particles, U32),
    PBF_SIM_FIELD("cube_layers", cube_layers, U32),
    PBF_SIM_FIELD("cube_group_spacing_world", cube_group_spacing_world, F32),
    PBF_SIM_FIELD("cube_layer_spacing_world", cube_layer_spacing_world, F32),
    PBF_SIM_FIELD("cube_base_height", cube_base_height, F32),
    PBF_SIM_FIELD("cube_lattice_spacing_factor_h", cube_lattice_spacing_factor_h, F32),
    PBF_SIM_FIELD("cube_initial_density", cube_initial_density, F32),
    PBF_SIM_FIELD("cube_auto_fit_domain", cube_auto_fit_domain, Bool),
    PBF_SIM_FIELD("cube_domain_margin_scale", cube_domain_margin_scale, F32),
    PBF_SIM_FIELD("cube_apply_initial_jitter", cube_apply_initial_jitter, Bool),
    PBF_SIM_FIELD("cube_layer_jitter_enable", cube_layer_jitter_enable, Bool),
    PBF_SIM_FIELD("cube_layer_jitter_scale_h", cube_layer_jitter_scale_h, F32),
    PBF_SIM_FIELD("cube_layer_jitter_seed", cube_layer_jitter_seed, U32),
    PBF_SIM_FIELD("cube_particles_per_group", cube_particles_per_group, U32),
    PBF_SIM_FIELD("integrate_semi_implicit", integrate_semi_implicit, Bool),
    PBF_SIM_FIELD("lambda_warm_start_enable", lambda_warm_start_enable, Bool),
    PBF_SIM_FIELD("lambda_warm_start_decay", lambda_warm_start_decay, F32),
    PBF_SIM_FIELD("xpbd_enable", xpbd_enable, Bool),
    PBF_SIM_FIELD("xpbd_compliance", xpbd_compliance, F32),
    PBF_SIM_FIELD("initial_jitter_enable", initial_jitter_enable, Bool),
    PBF_SIM_FIELD("initial_jitter_scale_h", initial_jitter_scale_h, F32),
    PBF_SIM_FIELD("initial_jitter_seed", initial_jitter_seed, U32),
    PBF_TUNING_FIELD(scorr_enable, I32),
    PBF_TUNING_FIELD(scorr_k, F32),
    PBF_TUNING_FIELD(scorr_n, F32),
    PBF_TUNING_FIELD(scorr_dq_h, F32),
    PBF_TUNING_FIELD(wq_min, F32),
    PBF_TUNING_FIELD(scorr_min, F32),
    PBF_TUNING_FIELD(grad_r_eps, F32),
    PBF_TUNING_FIELD(lambda_denom_eps, F32),
    PBF_TUNING_FIELD(compliance, F32),
    PBF_TUNING_FIELD(xpbd_enable, I32),
    PBF_TUNING_FIELD(enable_lambda_clamp, I32),
    PBF_TUNING_FIELD(lambda_max_abs, F32),
    PBF_TUNING_FIELD(enable_disp_clamp, I32),
    PBF_TUNING_FIELD(disp_clamp_max_h, F32),
    PBF_TUNING_FIELD(enable_relax, I32),
    PBF_TUNING_FIELD(relax_omega, F32),
    PBF_TUNING_FIELD(xsph_gate_enable, I32),
    PBF_TUNING_FIELD(xsph_n_min, I32),
    PBF_TUNING_FIELD(xsph_n_max, I32),
    PBF_TUNING_FIELD(lambda_warm_start_enable, I32),
    PBF_TUNING_FIELD(lambda_warm_start_decay, F32),
    PBF_TUNING_FIELD(semi_implicit_integration_enable, I32),
    PBF_PERF_FIELD("grid_cell_size_multiplier", grid_cell_size_multiplier, F32),
    PBF_PERF_FIELD("neighbor_cap", neighbor_cap, I32),
    PBF_PERF_FIELD("launch_bounds_tbs", launch_bounds_tbs, I32),
    PBF_PERF_FIELD("min_blocks_per_sm", min_blocks_per_sm, I32),
    PBF_PERF_FIELD("use_hashed_grid", use_hashed_grid, Bool),
    PBF_PERF_FIELD("sort_compact_every_n", sort_compact_every_n, I32),
    PBF_PERF_FIELD("compact_binary_search", compact_binary_search, Bool),
    PBF_PERF_FIELD("log_grid_compact_stats", log_grid_compact_stats, Bool),
};

#undef PBF_SIM_FIELD
#undef PBF_PERF_FIELD
#undef PBF_TUNING_FIELD

const Field* find_field(const char* name) {
    if (!name) return nullptr;
    for (const Field& f : kFields)
        if (std::strcmp(f.name, name) == 0) return &f;
    return nullptr;
}

}  // namespace

extern "C" {

int pbf_console_create(pbf_console** out) {
    if (!out) return PBF_ERR_INVALID;
    *out = new (std::nothrow) pbf_console;
    return *out ? PBF_OK : PBF_ERR_OOM;
}

int pbf_console_destroy(pbf_console* c) {
    delete c;
    return PBF_OK;
}

int pbf_console_set(pbf_console* c, const char* field, double value) {
    const Field* f = c ? find_field(field) : nullptr;
    if (!f || std::isnan(value)) return PBF_ERR_INVALID;
    void* p = f->at(c->c);
    switch (f->type) {
    case FieldType::F32: *static_cast<float*>(p) = float(value); break;
    case FieldType::I32:
        if (!(value >= double(INT_MIN) && value <= double(INT_MAX))) return PBF_ERR_INVALID;
        *static_cast<int*>(p) = int(value);
        break;
    case FieldType::U32:
        if (!(value >= 0.0 && value <= 4294967295.0)) return PBF_ERR_INVALID;
        *static_cast<uint32_t*>(p) = uint32_t(value);
        break;
    case FieldType::Bool: *static_cast<bool*>(p) = value != 0.0; break;
    case FieldType::MassMode:
        if (!(value == 0.0 || value == 1.0 || value == 2.0)) return PBF_ERR_INVALID;
        *static_cast<Sim::MassMode*>(p) = static_cast<Sim::MassMode>(uint32_t(value));
        break;
    }
    return PBF_OK;
}

int pbf_console_get(pbf_console* c, const char* field, double* value) {
    const Field* f = c ? find_field(field) : nullptr;
    if (!f || !value) return PBF_ERR_INVALID;
    void* p = f->at(c->c);
    switch (f->type) {
    case FieldType::F32: *value = *static_cast<float*>(p); break;
    case FieldType::I32: *value = *static_cast<int*>(p); break;
    case FieldType::U32: *value = *static_cast<uint32_t*>(p); break;
    case FieldType::Bool: *value = *static_cast<bool*>(p) ? 1.0 : 0.0; break;
    case FieldType::MassMode: *value = double(static_cast<uint32_t>(*static_cast<Sim::MassMode*>(p))); break;
    }
    return PBF_OK;
}

int pbf_console_prepare_cube_mix(pbf_console* c) {
    if (!c) return PBF_ERR_INVALID;
    console::PrepareCubeMix(c->c);
    return PBF_OK;
}

int pbf_console_merge_json(pbf_console* c, const char* text, char* err, uint32_t err_cap) {
    if (!c || !text) return PBF_ERR_INVALID;
    std::string e;
    if (!console::MergeConfigJson(c->c, text, &c->profile, &e)) {
        if (err && err_cap > 0) {
            const size_t n = std::min<size_t>(e.size(), err_cap - 1);
            std::memcpy(err, e.data(), n);
            err[n] = '\0';
        }
        return PBF_ERR_INVALID;
    }
    if (err && err_cap > 0) err[0] = '\0';
    return PBF_OK;
}

int pbf_console_profile(pbf_console* c, char* name, uint32_t cap) {
    if (!c || !name || cap == 0) return PBF_ERR_INVALID;
    if (c->profile.size() >= cap) return PBF_ERR_INVALID;
    std::memcpy(name, c->profile.c_str(), c->profile.size() + 1);
    return PBF_OK;
}

int pbf_console_build_sim_params(pbf_console* c, int sanitize, pbf_sim_params* out) {
    if (!c || !out) return PBF_ERR_INVALID;
    sim::SimParams sp{};
    console::BuildSimParams(c->c, sp);
    if (sanitize) console::SanitizeSimParams(c->c, sp);
    std::memcpy(out, &sp, sizeof(sp));
    return PBF_OK;
}

int pbf_console_cube_mix_centers(pbf_console* c, float* xyz, uint32_t cap, uint32_t* count) {
    if (!c || !count) return PBF_ERR_INVALID;
    std::vector<float3> centres;
    console::GenerateCubeMixCenters(c->c, centres);
    *count = uint32_t(centres.size());
    if (!xyz) return PBF_OK;
    if (cap < centres.size()) return PBF_ERR_INVALID;
    for (size_t i = 0; i < centres.size(); ++i) {
        xyz[3 * i] = centres[i].x;
        xyz[3 * i + 1] = centres[i].y;
        xyz[3 * i + 2] = centres[i].z;
    }
    return PBF_OK;
}

int pbf_seed_cube_mix(pbf_sim* h, pbf_console* c) {
    if (!h || !c) return PBF_ERR_INVALID;
    const Sim& s = c->c.sim;
    std::vector<float3> centres;
    console::GenerateCubeMixCenters(c->c, centres);
    const uint64_t total = uint64_t(s.cube_group_count) * s.cube_edge_particles * s.cube_edge_particles *
                           s.cube_edge_particles;
    if (centres.size() != s.cube_group_count || total != h->sim.activeParticleCount()) return PBF_ERR_INVALID;
    const float kh = h->sim.params().kernel.h;
    const float spacing = kh * ((s.cube_lattice_spacing_factor_h > 0.f) ? s.cube_lattice_spacing_factor_h : 1.0f);
    h->sim.seedCubeMix(s.cube_group_count, centres.data(), s.cube_edge_particles, spacing,
                       s.cube_apply_initial_jitter && s.initial_jitter_enable, s.initial_jitter_scale_h * kh,
                       s.initial_jitter_seed);
    return cudaGetLastError() == cudaSuccess ? PBF_OK : PBF_ERR_CUDA;
}

}  // extern "C"
