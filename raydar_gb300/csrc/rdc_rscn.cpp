// rdc_rscn.cpp -- the reference's .rscn scene format (serde JSON of
// src/scene/mod.rs:13-18) read into / written from rdc_scene_desc.
//
// Layout (src/scene/camera.rs:13-30, objects.rs:12-50, material.rs:4-13,
// world.rs:6-14): vectors are {"x","y","z"}; a Matrix4 is four column objects
// "x".."w" of {"x","y","z","w"} (column-major, as rdc_camera stores them);
// enums are externally tagged: {"Perspective":{"fov"}} | {"Orthographic":
// {"size"}}, {"SkyColor":{"top_color","bottom_color"}} | {"SolidColor":vec} |
// "Transparent", {"Sphere":{"center","radius"}} | {"Cube":{"center",
// "side_length"}}.  Numbers are read as f64 and rounded to f32, the
// conversion serde applies to f32 fields; matrices are taken as stored.
// Floats are written with the fewest digits that read back to the same f32.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "raydar_cuda.h"
#include "rdc_internal.hpp"

namespace {

struct Value {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;

    const Value* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

// Recursive-descent JSON reader (RFC 8259), depth-limited.
class Reader {
  public:
    Reader(const char* p, size_t n) : p_(p), end_(p + n) {}
    bool parse(Value& v, std::string& err) {
        if (!value(v, 0)) {
            err = err_.empty() ? "malformed JSON" : err_;
            return false;
        }
        ws();
        if (p_ != end_) {
            err = "trailing characters after the JSON value";
            return false;
        }
        return true;
    }

  private:
    const char* p_;
    const char* end_;
    std::string err_;

    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    bool lit(const char* s) {
        const size_t n = std::strlen(s);
        if ((size_t)(end_ - p_) < n || std::strncmp(p_, s, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool value(Value& v, int depth) {
        if (depth > 64) {
            err_ = "JSON nested too deeply";
            return false;
        }
        ws();
        if (p_ >= end_) return false;
        const char c = *p_;
        if (c == '{') return object(v, depth);
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v.kind = Value::Str;
            return string(v.str);
        }
        if (lit("true")) {
            v.kind = Value::Bool;
            v.b = true;
            return true;
        }
        if (lit("false")) {
            v.kind = Value::Bool;
            return true;
        }
        if (lit("null")) {
            v.kind = Value::Null;
            return true;
        }
        return number(v);
    }
    bool object(Value& v, int depth) {
        v.kind = Value::Obj;
        ++p_;
        ws();
        if (p_ < end_ && *p_ == '}') {
            ++p_;
            return true;
        }
        for (;;) {
            ws();
            std::string key;
            if (p_ >= end_ || *p_ != '"' || !string(key)) return false;
            ws();
            if (p_ >= end_ || *p_ != ':') return false;
            ++p_;
            Value item;
            if (!value(item, depth + 1)) return false;
            v.obj.emplace_back(std::move(key), std::move(item));
            ws();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == '}') {
                ++p_;
                return true;
            }
            return false;
        }
    }
    bool array(Value& v, int depth) {
        v.kind = Value::Arr;
        ++p_;
        ws();
        if (p_ < end_ && *p_ == ']') {
            ++p_;
            return true;
        }
        for (;;) {
            Value item;
            if (!value(item, depth + 1)) return false;
            v.arr.push_back(std::move(item));
            ws();
            if (p_ < end_ && *p_ == ',') {
                ++p_;
                continue;
            }
            if (p_ < end_ && *p_ == ']') {
                ++p_;
                return true;
            }
            return false;
        }
    }
    bool string(std::string& out) {
        ++p_;  // opening quote
        while (p_ < end_ && *p_ != '"') {
            if (*p_ == '\\') {
                if (++p_ >= end_) return false;
                const char e = *p_++;
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
                        if (end_ - p_ < 4) return false;
                        unsigned cp = 0;
                        for (int i = 0; i < 4; ++i) {
                            const char h = *p_++;
                            cp <<= 4;
                            if (h >= '0' && h <= '9') cp |= (unsigned)(h - '0');
                            else if (h >= 'a' && h <= 'f') cp |= (unsigned)(h - 'a' + 10);
                            else if (h >= 'A' && h <= 'F') cp |= (unsigned)(h - 'A' + 10);
                            else return false;
                        }
                        // keys and tags here are ASCII; keep other code points as UTF-8
                        if (cp < 0x80) {
                            out += (char)cp;
                        } else if (cp < 0x800) {
                            out += (char)(0xC0 | (cp >> 6));
                            out += (char)(0x80 | (cp & 0x3F));
                        } else {
                            out += (char)(0xE0 | (cp >> 12));
                            out += (char)(0x80 | ((cp >> 6) & 0x3F));
                            out += (char)(0x80 | (cp & 0x3F));
                        }
                        break;
                    }
                    default: return false;
                }
            } else {
                out += *p_++;
            }
        }
        if (p_ >= end_) return false;
        ++p_;  // closing quote
        return true;
    }
    bool number(Value& v) {
        const char* s = p_;
        if (p_ < end_ && *p_ == '-') ++p_;
        while (p_ < end_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '+' ||
                             *p_ == '-'))
            ++p_;
        if (p_ == s) return false;
        const std::string tok(s, p_);
        char* e = nullptr;
        errno = 0;
        v.num = std::strtod(tok.c_str(), &e);
        if (!e || *e != '\0') {
            err_ = "bad number '" + tok + "'";
            return false;
        }
        v.kind = Value::Num;
        return true;
    }
};

struct Fail {
    std::string msg;
};

float num(const Value* v, const char* what) {
    if (!v || v->kind != Value::Num) throw Fail{std::string("expected a number at ") + what};
    return (float)v->num;
}

void vec3(const Value* v, float out[3], const std::string& what) {
    if (!v || v->kind != Value::Obj) throw Fail{"expected a vector {x, y, z} at " + what};
    out[0] = num(v->get("x"), (what + ".x").c_str());
    out[1] = num(v->get("y"), (what + ".y").c_str());
    out[2] = num(v->get("z"), (what + ".z").c_str());
}

void mat4(const Value* v, float out[16], const std::string& what) {
    if (!v || v->kind != Value::Obj) throw Fail{"expected a matrix at " + what};
    const char* cols[4] = {"x", "y", "z", "w"};
    for (int c = 0; c < 4; ++c) {
        const Value* col = v->get(cols[c]);
        if (!col || col->kind != Value::Obj) throw Fail{"expected column " + std::string(cols[c]) + " at " + what};
        for (int r = 0; r < 4; ++r) out[4 * c + r] = num(col->get(cols[r]), (what + "." + cols[c]).c_str());
    }
}

uint32_t u32(const Value* v, const char* what) {
    if (!v || v->kind != Value::Num || v->num < 0 || v->num > 4294967295.0 || std::floor(v->num) != v->num)
        throw Fail{std::string("expected an unsigned integer at ") + what};
    return (uint32_t)v->num;
}

// The only key of an externally tagged enum object, or the string of a unit variant.
std::pair<std::string, const Value*> tag(const Value* v, const char* what) {
    if (v && v->kind == Value::Str) return {v->str, nullptr};
    if (!v || v->kind != Value::Obj || v->obj.size() != 1) throw Fail{std::string("expected an enum at ") + what};
    return {v->obj[0].first, &v->obj[0].second};
}

void read_camera(const Value* v, rdc_camera& c) {
    if (!v || v->kind != Value::Obj) throw Fail{"expected the camera object"};
    std::memset(&c, 0, sizeof(c));
    vec3(v->get("position"), c.position, "camera.position");
    vec3(v->get("target"), c.target, "camera.target");
    vec3(v->get("up"), c.up, "camera.up");
    c.resolution_x = u32(v->get("resolution_x"), "camera.resolution_x");
    c.resolution_y = u32(v->get("resolution_y"), "camera.resolution_y");
    const auto proj = tag(v->get("projection"), "camera.projection");
    if (proj.first == "Perspective" && proj.second) {
        c.projection = RDC_PROJECTION_PERSPECTIVE;
        c.fov_degrees = num(proj.second->get("fov"), "camera.projection.fov");
    } else if (proj.first == "Orthographic" && proj.second) {
        c.projection = RDC_PROJECTION_ORTHOGRAPHIC;
        c.ortho_size = num(proj.second->get("size"), "camera.projection.size");
    } else {
        throw Fail{"unknown projection '" + proj.first + "'"};
    }
    c.near_clip = num(v->get("near_clip"), "camera.near_clip");
    c.far_clip = num(v->get("far_clip"), "camera.far_clip");
    mat4(v->get("view_matrix"), c.view_matrix, "camera.view_matrix");
    mat4(v->get("proj_matrix"), c.proj_matrix, "camera.proj_matrix");
    mat4(v->get("inverse_view_matrix"), c.inverse_view_matrix, "camera.inverse_view_matrix");
    mat4(v->get("inverse_proj_matrix"), c.inverse_proj_matrix, "camera.inverse_proj_matrix");
}

void read_world(const Value* v, rdc_world& w) {
    std::memset(&w, 0, sizeof(w));
    const auto t = tag(v, "world");
    if (t.first == "SkyColor" && t.second) {
        w.kind = RDC_WORLD_SKY_COLOR;
        vec3(t.second->get("top_color"), w.top_color, "world.top_color");
        vec3(t.second->get("bottom_color"), w.bottom_color, "world.bottom_color");
    } else if (t.first == "SolidColor" && t.second) {
        w.kind = RDC_WORLD_SOLID_COLOR;
        vec3(t.second, w.solid_color, "world.SolidColor");
    } else if (t.first == "Transparent" && !t.second) {
        w.kind = RDC_WORLD_TRANSPARENT;
    } else {
        throw Fail{"unknown world '" + t.first + "'"};
    }
}

void read_object(const Value* v, rdc_object& o, size_t i) {
    const std::string at = "objects[" + std::to_string(i) + "]";
    if (!v || v->kind != Value::Obj) throw Fail{"expected an object at " + at};
    std::memset(&o, 0, sizeof(o));
    const auto g = tag(v->get("geometry"), (at + ".geometry").c_str());
    if (!g.second) throw Fail{"unknown geometry at " + at};
    vec3(g.second->get("center"), o.center, at + ".center");
    if (g.first == "Sphere") {
        o.geometry = RDC_GEOMETRY_SPHERE;
        o.radius = num(g.second->get("radius"), (at + ".radius").c_str());
    } else if (g.first == "Cube") {
        o.geometry = RDC_GEOMETRY_CUBE;
        o.side_length = num(g.second->get("side_length"), (at + ".side_length").c_str());
    } else {
        throw Fail{"unknown geometry '" + g.first + "' at " + at};
    }
    const Value* m = v->get("material");
    if (!m || m->kind != Value::Obj) throw Fail{"expected a material at " + at};
    rdc_material& mt = o.material;
    vec3(m->get("albedo"), mt.albedo, at + ".albedo");
    mt.roughness = num(m->get("roughness"), "roughness");
    mt.metallic = num(m->get("metallic"), "metallic");
    vec3(m->get("emission_color"), mt.emission_color, at + ".emission_color");
    mt.emission_strength = num(m->get("emission_strength"), "emission_strength");
    mt.transmission = num(m->get("transmission"), "transmission");
    mt.ior = num(m->get("ior"), "ior");
}

// Shortest decimal that reads back (f64 parse, f32 rounding) as the same f32.
void put_float(std::string& s, float f) {
    if (!std::isfinite(f)) throw Fail{"non-finite float cannot be written as JSON"};
    char buf[40];
    for (int p = 1; p <= 9; ++p) {
        std::snprintf(buf, sizeof(buf), "%.*g", p, (double)f);
        if ((float)std::strtod(buf, nullptr) == f) break;
    }
    s += buf;
    // serde writes floats with a decimal point or exponent (1.0, not 1)
    if (!std::strpbrk(buf, ".eEn")) s += ".0";
}

void put_vec3(std::string& s, const float v[3]) {
    s += "{\"x\":";
    put_float(s, v[0]);
    s += ",\"y\":";
    put_float(s, v[1]);
    s += ",\"z\":";
    put_float(s, v[2]);
    s += "}";
}

void put_mat4(std::string& s, const float m[16]) {
    const char* k[4] = {"x", "y", "z", "w"};
    s += "{";
    for (int c = 0; c < 4; ++c) {
        s += c ? ",\"" : "\"";
        s += k[c];
        s += "\":{";
        for (int r = 0; r < 4; ++r) {
            s += r ? ",\"" : "\"";
            s += k[r];
            s += "\":";
            put_float(s, m[4 * c + r]);
        }
        s += "}";
    }
    s += "}";
}

std::string write_scene(const rdc_scene_desc& d) {
    std::string s;
    const rdc_camera& c = d.camera;
    s += "{\"camera\":{\"position\":";
    put_vec3(s, c.position);
    s += ",\"target\":";
    put_vec3(s, c.target);
    s += ",\"up\":";
    put_vec3(s, c.up);
    s += ",\"resolution_x\":" + std::to_string(c.resolution_x);
    s += ",\"resolution_y\":" + std::to_string(c.resolution_y);
    if (c.projection == RDC_PROJECTION_PERSPECTIVE) {
        s += ",\"projection\":{\"Perspective\":{\"fov\":";
        put_float(s, c.fov_degrees);
    } else if (c.projection == RDC_PROJECTION_ORTHOGRAPHIC) {
        s += ",\"projection\":{\"Orthographic\":{\"size\":";
        put_float(s, c.ortho_size);
    } else {
        throw Fail{"unknown projection kind"};
    }
    s += "}},\"near_clip\":";
    put_float(s, c.near_clip);
    s += ",\"far_clip\":";
    put_float(s, c.far_clip);
    s += ",\"view_matrix\":";
    put_mat4(s, c.view_matrix);
    s += ",\"proj_matrix\":";
    put_mat4(s, c.proj_matrix);
    s += ",\"inverse_view_matrix\":";
    put_mat4(s, c.inverse_view_matrix);
    s += ",\"inverse_proj_matrix\":";
    put_mat4(s, c.inverse_proj_matrix);
    s += "},\"world\":";
    const rdc_world& w = d.world;
    if (w.kind == RDC_WORLD_SKY_COLOR) {
        s += "{\"SkyColor\":{\"top_color\":";
        put_vec3(s, w.top_color);
        s += ",\"bottom_color\":";
        put_vec3(s, w.bottom_color);
        s += "}}";
    } else if (w.kind == RDC_WORLD_SOLID_COLOR) {
        s += "{\"SolidColor\":";
        put_vec3(s, w.solid_color);
        s += "}";
    } else if (w.kind == RDC_WORLD_TRANSPARENT) {
        s += "\"Transparent\"";
    } else {
        throw Fail{"unknown world kind"};
    }
    s += ",\"objects\":[";
    for (uint32_t i = 0; i < d.object_count; ++i) {
        const rdc_object& o = d.objects[i];
        s += i ? ",{\"geometry\":" : "{\"geometry\":";
        if (o.geometry == RDC_GEOMETRY_SPHERE) {
            s += "{\"Sphere\":{\"center\":";
            put_vec3(s, o.center);
            s += ",\"radius\":";
            put_float(s, o.radius);
        } else if (o.geometry == RDC_GEOMETRY_CUBE) {
            s += "{\"Cube\":{\"center\":";
            put_vec3(s, o.center);
            s += ",\"side_length\":";
            put_float(s, o.side_length);
        } else {
            throw Fail{"unknown geometry kind at object " + std::to_string(i)};
        }
        const rdc_material& m = o.material;
        s += "}},\"material\":{\"albedo\":";
        put_vec3(s, m.albedo);
        s += ",\"roughness\":";
        put_float(s, m.roughness);
        s += ",\"metallic\":";
        put_float(s, m.metallic);
        s += ",\"emission_color\":";
        put_vec3(s, m.emission_color);
        s += ",\"emission_strength\":";
        put_float(s, m.emission_strength);
        s += ",\"transmission\":";
        put_float(s, m.transmission);
        s += ",\"ior\":";
        put_float(s, m.ior);
        s += "}}";
    }
    s += "]}";
    return s;
}

}  // namespace

extern "C" {

rdc_status rdc_scene_parse_rscn(const char* text, size_t length, rdc_scene_desc* scene_out, rdc_object* objects_out,
                                uint32_t capacity, uint32_t* count_out) {
    if (!text || !scene_out || !count_out) {
        rdc::set_thread_error("rdc_scene_parse_rscn: NULL argument");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    Value root;
    std::string err;
    if (!Reader(text, length).parse(root, err)) {
        rdc::set_thread_error("rdc_scene_parse_rscn: " + err);
        return RDC_ERR_INVALID_ARGUMENT;
    }
    try {
        if (root.kind != Value::Obj) throw Fail{"the scene is not a JSON object"};
        const Value* objs = root.get("objects");
        if (!objs || objs->kind != Value::Arr) throw Fail{"expected the objects array"};
        if (objs->arr.size() > RDC_MAX_OBJECTS) {
            rdc::set_thread_error("rdc_scene_parse_rscn: more than RDC_MAX_OBJECTS objects");
            return RDC_ERR_LIMIT;
        }
        rdc_scene_desc d;
        std::memset(&d, 0, sizeof(d));
        read_camera(root.get("camera"), d.camera);
        read_world(root.get("world"), d.world);
        const uint32_t n = (uint32_t)objs->arr.size();
        *count_out = n;
        if (objects_out && capacity >= n) {
            for (uint32_t i = 0; i < n; ++i) read_object(&objs->arr[i], objects_out[i], i);
        } else if (objects_out || capacity) {
            rdc::set_thread_error("rdc_scene_parse_rscn: capacity below the object count (*count_out)");
            return RDC_ERR_LIMIT;
        } else {
            // size query: still validate every object
            rdc_object tmp;
            for (uint32_t i = 0; i < n; ++i) read_object(&objs->arr[i], tmp, i);
        }
        d.objects = objects_out;
        d.object_count = (objects_out && capacity >= n) ? n : 0;
        *scene_out = d;
    } catch (const Fail& f) {
        rdc::set_thread_error("rdc_scene_parse_rscn: " + f.msg);
        return RDC_ERR_INVALID_ARGUMENT;
    }
    return RDC_OK;
}

rdc_status rdc_scene_write_rscn(const rdc_scene_desc* scene, char* buf, size_t capacity, size_t* length_out) {
    if (!scene || !length_out || (scene->object_count && !scene->objects)) {
        rdc::set_thread_error("rdc_scene_write_rscn: NULL argument");
        return RDC_ERR_INVALID_ARGUMENT;
    }
    std::string s;
    try {
        s = write_scene(*scene);
    } catch (const Fail& f) {
        rdc::set_thread_error("rdc_scene_write_rscn: " + f.msg);
        return RDC_ERR_INVALID_ARGUMENT;
    }
    *length_out = s.size();
    if (!buf) return RDC_OK;
    if (capacity < s.size() + 1) {
        rdc::set_thread_error("rdc_scene_write_rscn: buffer smaller than *length_out + 1");
        return RDC_ERR_LIMIT;
    }
    std::memcpy(buf, s.c_str(), s.size() + 1);
    return RDC_OK;
}

}  // extern "C"
