// scene.cpp — scene JSON loader, physical parameters and the initial lattice.
//
// Host-only code; no CUDA call is made here, so all of it is testable without
// a GPU. Behaviour follows the reference:
//   readSceneFromJsonFile        src/simulation/sph_hybrid_system.cpp:69-126
//   defaultInitializeSPHSysPara  src/simulation/sph_hybrid_system.cpp:127-202
//   initializeScene (lattice)    src/simulation/sph_hybrid_system.cpp:432-473
// The reference reads JSON through jsoncpp; this file carries its own small
// JSON reader for the same keys (objects, arrays, numbers, strings, literals).
#define _USE_MATH_DEFINES
#include <cerrno>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gsph_internal.h"

namespace gsph {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

namespace {

// ---------------------------------------------------------------- JSON ----
struct JVal {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<JVal> arr;
    std::vector<std::pair<std::string, JVal>> obj;
    const JVal *get(const char *k) const {
        if (kind != Obj) return nullptr;
        for (const auto &kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

class JParser {
  public:
    JParser(const char *s, size_t n) : p_(s), end_(s + n) {}
    bool parse(JVal &out) {
        ws();
        if (!value(out, 0)) return false;
        ws();
        if (p_ != end_) return fail("trailing characters");
        return true;
    }
    const char *error() const { return err_; }
    size_t offset(const char *base) const { return size_t(p_ - base); }

  private:
    const char *p_, *end_;
    const char *err_ = "";
    bool fail(const char *m) {
        err_ = m;
        return false;
    }
    void ws() {
        while (p_ < end_) {
            if (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r') {
                ++p_;
            } else if (*p_ == '/' && p_ + 1 < end_ && p_[1] == '/') {
                while (p_ < end_ && *p_ != '\n') ++p_;   // jsoncpp accepts comments
            } else if (*p_ == '/' && p_ + 1 < end_ && p_[1] == '*') {
                p_ += 2;
                while (p_ + 1 < end_ && !(p_[0] == '*' && p_[1] == '/')) ++p_;
                p_ = (p_ + 1 < end_) ? p_ + 2 : end_;
            } else {
                break;
            }
        }
    }
    bool lit(const char *w) {
        size_t n = std::strlen(w);
        if (size_t(end_ - p_) < n || std::memcmp(p_, w, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool string(std::string &s) {
        if (p_ >= end_ || *p_ != '"') return fail("expected string");
        ++p_;
        while (p_ < end_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= end_) return fail("bad escape");
                char e = *p_++;
                switch (e) {
                    case 'n': s += '\n'; break;
                    case 't': s += '\t'; break;
                    case 'r': s += '\r'; break;
                    case 'b': s += '\b'; break;
                    case 'f': s += '\f'; break;
                    case 'u':
                        if (end_ - p_ < 4) return fail("bad \\u escape");
                        p_ += 4;
                        s += '?';
                        break;
                    default: s += e; break;
                }
            } else {
                s += c;
            }
        }
        if (p_ >= end_) return fail("unterminated string");
        ++p_;
        return true;
    }
    bool value(JVal &v, int depth) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (p_ >= end_) return fail("unexpected end of input");
        char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = JVal::Obj;
            ws();
            if (p_ < end_ && *p_ == '}') { ++p_; return true; }
            for (;;) {
                ws();
                std::string k;
                if (!string(k)) return false;
                ws();
                if (p_ >= end_ || *p_ != ':') return fail("expected ':'");
                ++p_;
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.obj.emplace_back(std::move(k), std::move(child));
                ws();
                if (p_ < end_ && *p_ == ',') { ++p_; continue; }
                if (p_ < end_ && *p_ == '}') { ++p_; return true; }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++p_;
            v.kind = JVal::Arr;
            ws();
            if (p_ < end_ && *p_ == ']') { ++p_; return true; }
            for (;;) {
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.arr.push_back(std::move(child));
                ws();
                if (p_ < end_ && *p_ == ',') { ++p_; continue; }
                if (p_ < end_ && *p_ == ']') { ++p_; return true; }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = JVal::Str;
            return string(v.str);
        }
        if (lit("true")) { v.kind = JVal::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = JVal::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = JVal::Null; return true; }
        if (c == '-' || c == '+' || (c >= '0' && c <= '9') || c == '.') {
            std::string tok;
            while (p_ < end_ && (std::strchr("+-0123456789.eE", *p_) != nullptr))
                tok += *p_++;
            char *e = nullptr;
            errno = 0;
            v.num = std::strtod(tok.c_str(), &e);
            if (e == tok.c_str() || *e != '\0') return fail("bad number");
            v.kind = JVal::Num;
            return true;
        }
        return fail("unexpected character");
    }
};

// jsoncpp's asFloat()/asUInt() on numbers, bools and null.
bool as_double(const JVal *v, double &out) {
    if (!v) return false;
    if (v->kind == JVal::Num) { out = v->num; return true; }
    if (v->kind == JVal::Bool) { out = v->b ? 1.0 : 0.0; return true; }
    if (v->kind == JVal::Null) { out = 0.0; return true; }
    return false;
}

}  // namespace

// SplitMix64 (Steele, Lea, Flood 2014; Vigna's public-domain reference).
static inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Uniform jitter in [-1, 1) for (seed, particle, axis).
static inline double jitter_unit(uint64_t seed, uint64_t particle, int axis) {
    uint64_t z = splitmix64(seed * 0x632BE59BD9B4E019ull + particle * 3ull +
                            uint64_t(axis));
    return double(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

DevParams make_dev_params(const gsph_params &p) {
    DevParams d{};
    d.h = p.kernel;
    d.h2 = p.kernel_2;
    d.rat = 4.f * p.inv_cell_size;   // sph_utils.cuh:48 "4.f * inv_cell_size"
    d.numc = p.grid_size[0] * p.grid_size[1] * p.grid_size[2];
    d.density_scale = p.density_scale;
    d.self_density = p.self_density;
    d.rest_density = p.rest_density;
    d.inv_rest_density = p.inv_rest_density;
    d.gas_constant = p.gas_constant;
    d.half_spiky = p.half_spiky_value;
    d.visco_coef = p.viscosity_visco_value;
    d.grad_color_scale = p.grad_color_scale;
    d.lplc_color_scale = p.lplc_color_scale;
    d.surface_normal = p.surface_normal;
    d.surface_coe = p.surface_coe;
    d.mass = p.mass;
    d.time_step = p.time_step;
    d.wall_damping = p.wall_damping;
    // integration_kernels.cu:253 "kDevSysPara.kernel + 0.01" is a double sum
    // rounded to float.
    d.wall_kernel = float(double(p.kernel) + 0.01);
    d.gx_acc = p.gravity[0];
    d.gy_acc = p.gravity[1];
    d.gz_acc = p.gravity[2];
    d.bmin = p.bound_min[0];
    d.visc_artificial = 0;
    d.art_coef = 0.f;
    d.art_eps = 0.01f * p.kernel_2;
    d.spiky = p.spiky_value;
    d.sparse_total = 96;   // gpu_model.cu:172-180
    d.sparse_self = 15;
    d.mid_total = 60;
    return d;
}

gsph_status check_grid(const gsph_params &p, const char *who, long long *numc) {
    for (int a = 0; a < 3; ++a) {
        if (p.grid_size[a] < 1 || p.grid_size[a] > 65535) {
            set_error("%s: grid size %d along axis %d out of range [1, 65535]",
                      who, int(p.grid_size[a]), a);
            return GSPH_ERR_INVALID_ARG;
        }
    }
    const long long c =
        (long long)p.grid_size[0] * p.grid_size[1] * p.grid_size[2];
    if (c >= kMaxCells) {
        set_error("%s: grid has %lld cells; at most 2^26 - 1 are supported", who, c);
        return GSPH_ERR_CAPACITY;
    }
    if (numc) *numc = c;
    return GSPH_OK;
}

SceneGeom make_scene_geom(const gsph_params &p, int cbase) {
    SceneGeom g{};
    g.gx = p.grid_size[0];
    g.gy = p.grid_size[1];
    g.gz = p.grid_size[2];
    g.cbase = cbase;
    g.bmax_x = p.bound_max[0];
    g.bmax_y = p.bound_max[1];
    g.bmax_z = p.bound_max[2];
    return g;
}

}  // namespace gsph

using namespace gsph;

extern "C" {

const char *gsph_last_error(void) { return g_err; }

int gsph_abi_version(void) { return GSPH_ABI_VERSION; }

gsph_status gsph_scene_default(gsph_scene *out) {
    if (!out) {
        set_error("gsph_scene_default: null output");
        return GSPH_ERR_INVALID_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    // Scene defaults, sph_hybrid_system.h:37-44.
    out->interval = 0.5f;
    out->mass = 0.02f;
    out->recomm_nump = 65536u;
    const float nan = std::nanf("");
    out->kernel = nan;
    out->rest_density = nan;
    out->gas_constant = nan;
    out->viscosity = nan;
    out->time_step = nan;
    out->gravity_y = nan;
    out->jitter = 0.f;
    out->seed = 0;
    return GSPH_OK;
}

gsph_status gsph_scene_parse_json(const char *text, size_t len,
                                  gsph_scene *out) {
    if (!text || !out) {
        set_error("gsph_scene_parse_json: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_scene s;
    gsph_scene_default(&s);
    JVal root;
    JParser parser(text, len);
    if (!parser.parse(root)) {
        set_error("can not parse scene: %s at offset %zu", parser.error(),
                  parser.offset(text));
        return GSPH_ERR_PARSE;
    }
    if (root.kind != JVal::Obj) {
        set_error("can not parse scene: top level is not an object");
        return GSPH_ERR_PARSE;
    }
    double d;
    auto num = [&](const char *k, float &dst) -> gsph_status {
        const JVal *v = root.get(k);
        if (!v) return GSPH_OK;
        if (!as_double(v, d)) {
            set_error("scene key \"%s\" is not a number", k);
            return GSPH_ERR_PARSE;
        }
        dst = float(d);
        return GSPH_OK;
    };
    gsph_status st;
    if ((st = num("xx", s.world[0])) || (st = num("yy", s.world[1])) ||
        (st = num("zz", s.world[2])) || (st = num("mass", s.mass)) ||
        (st = num("interval", s.interval)) || (st = num("kernel", s.kernel)) ||
        (st = num("rest_density", s.rest_density)) ||
        (st = num("gas_constant", s.gas_constant)) ||
        (st = num("viscosity", s.viscosity)) ||
        (st = num("time_step", s.time_step)) ||
        (st = num("gravity_y", s.gravity_y)) || (st = num("jitter", s.jitter)))
        return st;
    if (const JVal *v = root.get("recomm_nump")) {
        if (!as_double(v, d) || d < 0) {
            set_error("scene key \"recomm_nump\" is not an unsigned number");
            return GSPH_ERR_PARSE;
        }
        s.recomm_nump = uint32_t(d);
    }
    if (const JVal *v = root.get("seed")) {
        if (!as_double(v, d) || d < 0) {
            set_error("scene key \"seed\" is not an unsigned number");
            return GSPH_ERR_PARSE;
        }
        s.seed = uint64_t(d);
    }
    if (const JVal *fb = root.get("fluid_block")) {
        if (fb->kind != JVal::Arr) {
            set_error("scene key \"fluid_block\" is not an array");
            return GSPH_ERR_PARSE;
        }
        if (fb->arr.size() > GSPH_MAX_FLUID_BLOCKS) {
            set_error("scene has %zu fluid blocks (max %d)", fb->arr.size(),
                      GSPH_MAX_FLUID_BLOCKS);
            return GSPH_ERR_CAPACITY;
        }
        static const char *kb[3] = {"begin_x", "begin_y", "begin_z"};
        static const char *ke[3] = {"end_x", "end_y", "end_z"};
        for (size_t i = 0; i < fb->arr.size(); ++i) {
            const JVal &blk = fb->arr[i];
            for (int a = 0; a < 3; ++a) {
                // jsoncpp returns 0 for a missing member (Value::null).
                double b = 0.0, e = 0.0;
                const JVal *vb = blk.get(kb[a]);
                const JVal *ve = blk.get(ke[a]);
                if ((vb && !as_double(vb, b)) || (ve && !as_double(ve, e))) {
                    set_error("fluid_block[%zu] bound is not a number", i);
                    return GSPH_ERR_PARSE;
                }
                s.block_begin[i][a] = float(b);
                s.block_end[i][a] = float(e);
            }
        }
        s.n_blocks = uint32_t(fb->arr.size());
    }
    *out = s;
    return GSPH_OK;
}

gsph_status gsph_scene_load_json(const char *path, gsph_scene *out) {
    if (!path || !out) {
        set_error("gsph_scene_load_json: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error("can not open %s", path);
        return GSPH_ERR_IO;
    }
    std::string text;
    char buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
    std::fclose(f);
    gsph_status st = gsph_scene_parse_json(text.data(), text.size(), out);
    if (st == GSPH_ERR_PARSE) {
        std::string m = std::string(gsph_last_error()) + " (" + path + ")";
        set_error("%s", m.c_str());
    }
    return st;
}

gsph_status gsph_params_init(const gsph_scene *scene, gsph_params *out) {
    if (!scene || !out) {
        set_error("gsph_params_init: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_params p;
    std::memset(&p, 0, sizeof(p));
    // The arithmetic below keeps the reference's float/double mix
    // (sph_hybrid_system.cpp:136-193) so that every coefficient rounds the
    // same way.
    p.kernel = std::isnan(scene->kernel) ? 0.03f : scene->kernel;
    p.mass = scene->mass;
    p.kernel_2 = p.kernel * p.kernel;
    p.world_size[0] = scene->world[0];
    p.world_size[1] = scene->world[1];
    p.world_size[2] = scene->world[2];
    p.cell_size = p.kernel;
    p.inv_cell_size = 1.0f / p.cell_size;
    for (int a = 0; a < 3; ++a) {
        float g = std::ceil(p.world_size[a] / p.cell_size);
        if (!(g >= 1.f) || g > 65535.f) {
            set_error("grid size %g along axis %d out of range [1, 65535]",
                      double(g), a);
            return GSPH_ERR_INVALID_ARG;
        }
        p.grid_size[a] = int32_t(g);
    }
    const double numc = double(p.grid_size[0]) * p.grid_size[1] * p.grid_size[2];
    if (numc >= 67108864.0) {   // 32-bit micro keys need numc * 64 < 2^32
        set_error("grid has %.0f cells; at most 2^26 are supported", numc);
        return GSPH_ERR_CAPACITY;
    }
    p.gravity[0] = 0.0f;
    p.gravity[1] = std::isnan(scene->gravity_y) ? -9.8f : scene->gravity_y;
    p.gravity[2] = 0.0f;
    p.wall_damping = -0.5f;
    p.rest_density =
        std::isnan(scene->rest_density) ? 1000.0f : scene->rest_density;
    p.gas_constant =
        std::isnan(scene->gas_constant) ? 1.0f : scene->gas_constant;
    p.viscosity = std::isnan(scene->viscosity) ? 6.5f : scene->viscosity;
    p.time_step = std::isnan(scene->time_step) ? 0.003f : scene->time_step;
    p.surface_normal = 0.1f;
    p.surface_coe = 0.2f;
    const double kd = double(p.kernel);
    p.poly6_value = float(315.0f / (64.0f * M_PI * std::pow(kd, 9)));
    p.spiky_value = float(-45.0f / (M_PI * std::pow(kd, 6)));
    p.visco_value = float(45.0f / (M_PI * std::pow(kd, 6)));
    p.grad_poly6 = float(-945 / (32 * M_PI * std::pow(kd, 9)));
    p.lplc_poly6 = float(945 / (8 * M_PI * std::pow(kd, 9)));
    p.self_density = float(double(p.mass * p.poly6_value) * std::pow(kd, 6));
    p.inv_rest_density = 1.0f / p.rest_density;
    p.density_scale = p.mass * p.poly6_value;
    p.half_spiky_value = p.spiky_value * 0.5f;
    p.viscosity_visco_value = p.viscosity * p.visco_value;
    p.grad_color_scale = p.grad_poly6 * p.mass;
    p.lplc_color_scale = p.lplc_poly6 * p.mass;
    p.bound_interval = p.kernel;
    for (int a = 0; a < 3; ++a) {
        p.bound_min[a] = p.bound_interval;
        p.bound_max[a] = p.world_size[a] - p.bound_interval;
    }
    *out = p;
    return GSPH_OK;
}

// Lattice of initializeScene (sph_hybrid_system.cpp:441-464): for every fluid
// block, x outer, y middle, z inner, each coordinate advanced by FP32
// accumulation of kernel*interval while below the block end.
static gsph_status lattice_walk(const gsph_scene *s, const gsph_params *p,
                                float *pos4, uint32_t capacity,
                                uint32_t *count) {
    if (!s || !p || !count) {
        set_error("gsph_lattice: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    const float step = p->kernel * s->interval;
    if (!(step > 0.f)) {
        set_error("lattice step kernel*interval = %g is not positive",
                  double(step));
        return GSPH_ERR_INVALID_ARG;
    }
    const double jit = double(s->jitter) * double(step);
    uint64_t n = 0;
    for (uint32_t b = 0; b < s->n_blocks; ++b) {
        const float *lo = s->block_begin[b];
        const float *hi = s->block_end[b];
        for (float x = lo[0]; x < hi[0]; x += step)
            for (float y = lo[1]; y < hi[1]; y += step)
                for (float z = lo[2]; z < hi[2]; z += step) {
                    if (pos4) {
                        if (n >= capacity) {
                            set_error("lattice has more than %u particles",
                                      capacity);
                            return GSPH_ERR_CAPACITY;
                        }
                        float px = x, py = y, pz = z;
                        if (jit != 0.0) {
                            px = float(double(x) + jit * jitter_unit(s->seed, n, 0));
                            py = float(double(y) + jit * jitter_unit(s->seed, n, 1));
                            pz = float(double(z) + jit * jitter_unit(s->seed, n, 2));
                        }
                        pos4[4 * n + 0] = px;
                        pos4[4 * n + 1] = py;
                        pos4[4 * n + 2] = pz;
                        pos4[4 * n + 3] = 0.f;
                    }
                    if (++n > 0x7FFFFFFFull) {
                        set_error("lattice exceeds 2^31 particles");
                        return GSPH_ERR_CAPACITY;
                    }
                }
    }
    *count = uint32_t(n);
    return GSPH_OK;
}

gsph_status gsph_lattice_count(const gsph_scene *scene, const gsph_params *p,
                               uint32_t *count) {
    return lattice_walk(scene, p, nullptr, 0, count);
}

gsph_status gsph_lattice_fill(const gsph_scene *scene, const gsph_params *p,
                              float *pos4, uint32_t capacity, uint32_t *count) {
    if (!pos4) {
        set_error("gsph_lattice_fill: null output");
        return GSPH_ERR_INVALID_ARG;
    }
    return lattice_walk(scene, p, pos4, capacity, count);
}

}  // extern "C"
