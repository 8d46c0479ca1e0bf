// Lumen JSON + OBJ scene loading onto the arrays of include/lgb.h. See lumen_scene.h.
#include "lumen_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "json.h"
#include "mitsuba_xml.h"

namespace lgbh {
namespace {

std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string dir_of(const std::string& path) {
    const size_t p = path.find_last_of("/\\");
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

lgb_material default_material() {
    lgb_material m;
    std::memset(&m, 0, sizeof(m));
    m.texture_id = -1;
    return m;
}

void vec3_of(const Json& j, float* out, const float* def) {
    for (int i = 0; i < 3; i++) out[i] = j.is_null() ? def[i] : (float)j[i].as_number();
}

// One OBJ face corner: position / texcoord / normal indices (0-based, -1 = absent).
struct Corner {
    long v = -1, t = -1, n = -1;
};

long obj_index(const std::string& tok, size_t count) {
    if (tok.empty()) return -1;
    long i = std::strtol(tok.c_str(), nullptr, 10);
    if (i > 0) return i - 1;
    if (i < 0) return (long)count + i;
    return -1;
}

// reflectance_to_conductor_eta_k (LumenScene.cpp:47-50): eta = 1, k = 2 sqrt(r) / sqrt(max(1 - r, 0.001)), with
// r clamped to [0, 0.9999].
void conductor_from_reflectance(const float refl[3], lgb_material& m) {
    for (int a = 0; a < 3; a++) {
        const float r = std::min(std::max(refl[a], 0.0f), 0.9999f);
        m.albedo[a] = 1.0f;
        m.k[a] = 2.0f * std::sqrt(r) / std::sqrt(std::max(1.0f - r, 0.001f));
    }
}

}  // namespace

// OBJ subset of the files Lumen's scenes reference: v / vt / vn / f (polygons split into fans), with shapes
// started by 'o' or 'g'. Every face corner becomes its own vertex, as LumenScene.cpp:302-324 lays them out.
// Files without normals get the triangle's geometric normal (Lumen would read past its normal array) and
// files without texture coordinates get (0, 0).
void LumenScene::load_obj(const std::string& path) {
    std::istringstream in(read_file(path));
    std::vector<float> v, vt, vn;
    struct Shape {
        std::string name;
        std::vector<Corner> corners;  // 3 per triangle
    };
    std::vector<Shape> shapes(1);
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        std::istringstream ls(line);
        std::string tag;
        if (!(ls >> tag)) continue;
        if (tag == "v") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            v.push_back(x); v.push_back(y); v.push_back(z);
        } else if (tag == "vt") {
            float s = 0, t = 0;
            ls >> s >> t;
            vt.push_back(s); vt.push_back(t);
        } else if (tag == "vn") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            vn.push_back(x); vn.push_back(y); vn.push_back(z);
        } else if (tag == "o" || tag == "g") {
            std::string name;
            std::getline(ls, name);
            name.erase(0, name.find_first_not_of(" \t"));
            if (!shapes.back().corners.empty() || !shapes.back().name.empty()) shapes.emplace_back();
            shapes.back().name = name;
        } else if (tag == "f") {
            std::vector<Corner> poly;
            std::string tok;
            while (ls >> tok) {
                Corner c;
                size_t a = tok.find('/');
                if (a == std::string::npos) {
                    c.v = obj_index(tok, v.size() / 3);
                } else {
                    c.v = obj_index(tok.substr(0, a), v.size() / 3);
                    size_t b = tok.find('/', a + 1);
                    if (b == std::string::npos) {
                        c.t = obj_index(tok.substr(a + 1), vt.size() / 2);
                    } else {
                        c.t = obj_index(tok.substr(a + 1, b - a - 1), vt.size() / 2);
                        c.n = obj_index(tok.substr(b + 1), vn.size() / 3);
                    }
                }
                if (c.v < 0 || (size_t)c.v >= v.size() / 3) throw std::runtime_error("OBJ face index out of range in " + path);
                poly.push_back(c);
            }
            for (size_t k = 2; k < poly.size(); k++) {
                shapes.back().corners.push_back(poly[0]);
                shapes.back().corners.push_back(poly[k - 1]);
                shapes.back().corners.push_back(poly[k]);
            }
        }
    }
    for (const Shape& sh : shapes) {
        if (sh.corners.empty()) continue;
        lgb_mesh m;
        m.index_offset = (uint32_t)indices.size();
        m.vertex_offset = (uint32_t)(positions.size() / 3);
        m.material_index = 0;
        m.tri_count = (uint32_t)(sh.corners.size() / 3);
        for (size_t i = 0; i < sh.corners.size(); i += 3) {
            float fn[3] = {0, 0, 1};
            {
                const float* p0 = &v[3 * sh.corners[i].v];
                const float* p1 = &v[3 * sh.corners[i + 1].v];
                const float* p2 = &v[3 * sh.corners[i + 2].v];
                const float e0[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                const float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                const float c[3] = {e0[1] * e1[2] - e1[1] * e0[2], e0[2] * e1[0] - e1[2] * e0[0], e0[0] * e1[1] - e1[0] * e0[1]};
                const float l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
                if (l > 0) { fn[0] = c[0] / l; fn[1] = c[1] / l; fn[2] = c[2] / l; }
            }
            for (int k = 0; k < 3; k++) {
                const Corner& c = sh.corners[i + k];
                for (int a = 0; a < 3; a++) positions.push_back(v[3 * c.v + a]);
                for (int a = 0; a < 3; a++) normals.push_back(c.n >= 0 && (size_t)c.n < vn.size() / 3 ? vn[3 * c.n + a] : fn[a]);
                for (int a = 0; a < 2; a++) uvs.push_back(c.t >= 0 && (size_t)c.t < vt.size() / 2 ? vt[2 * c.t + a] : 0.0f);
                indices.push_back((uint32_t)(i + k));  // per-mesh local index (LumenScene.cpp:305)
            }
        }
        meshes.push_back(m);
        mesh_names.push_back(sh.name);
    }
}

void LumenScene::load(const std::string& path) {
    if (path.size() >= 4 && path.compare(path.size() - 4, 4, ".xml") == 0) load_mitsuba(path);
    else load_json(path);
}

void LumenScene::load_json(const std::string& json_path) {
    const Json j = parse_json(read_file(json_path));
    const std::string root = dir_of(json_path);
    // integrator block (LumenScene.cpp:237-247)
    const Json& integ = j["integrator"];
    if (!integ["type"].is_null()) {
        config.integrator = integ["type"].as_string();
        std::transform(config.integrator.begin(), config.integrator.end(), config.integrator.begin(), ::tolower);
    }
    if (!integ["path_length"].is_null()) config.path_length = (int)integ["path_length"].as_number();
    if (config.integrator == "sppm") {  // LumenScene.cpp:248-249
        if (!integ["base_radius"].is_null()) config.base_radius = (float)integ["base_radius"].as_number();
    } else if (config.integrator == "vcm") {  // LumenScene.cpp:250-253
        if (!integ["enable_vm"].is_null()) config.enable_vm = integ["enable_vm"].as_number() == 1;
        if (!integ["radius_factor"].is_null()) config.radius_factor = (float)integ["radius_factor"].as_number();
    }
    if (!integ["sky_col"].is_null()) vec3_of(integ["sky_col"], config.sky_col, config.sky_col);
    // geometry
    if (j["mesh_file"].is_null()) throw std::runtime_error("scene has no mesh_file");
    load_obj(root + j["mesh_file"].as_string());
    // materials (LumenScene.cpp:347-486)
    const Json& bsdfs = j["bsdfs"];
    materials.assign(std::max<size_t>(bsdfs.size(), 1), default_material());
    for (size_t bi = 0; bi < bsdfs.size(); bi++) {
        const Json& b = bsdfs[bi];
        lgb_material& m = materials[bi];
        const float one[3] = {1, 1, 1}, zero[3] = {0, 0, 0};
        if (!b["texture"].is_null()) {
            const std::string tex = root + b["texture"].as_string();
            if (tex.size() >= 4 && tex.compare(tex.size() - 4, 4, ".pfm") == 0) {
                textures.push_back(read_pfm(tex));
                m.texture_id = (int)textures.size() - 1;
            } else {
                std::fprintf(stderr, "lgbh: texture %s skipped (only PFM textures are read)\n", tex.c_str());
            }
        }
        vec3_of(b["albedo"], m.albedo, one);
        vec3_of(b["emissive_factor"], m.emissive_factor, zero);
        const std::string type = b["type"].is_null() ? std::string() : b["type"].as_string();
        if (type == "diffuse") {
            m.bsdf_type = LGB_BSDF_DIFFUSE;
            m.bsdf_props = LGB_FLAG_DIFFUSE | LGB_FLAG_REFLECTION;
        } else if (type == "mirror") {
            m.bsdf_type = LGB_BSDF_MIRROR;
            m.bsdf_props = LGB_FLAG_SPECULAR | LGB_FLAG_REFLECTION;
        } else if (type == "glass") {
            m.bsdf_type = LGB_BSDF_GLASS;
            m.bsdf_props = LGB_FLAG_SPECULAR | LGB_FLAG_TRANSMISSION;
            m.ior = b["ior"].f(1.0f);
        } else if (type == "dielectric") {
            m.bsdf_type = LGB_BSDF_DIELECTRIC;
            m.ior = b["ior"].f(1.0f);
            m.roughness = b["roughness"].f(0.0f);
            if (b["transmission"].is_null() || b["transmission"].as_number() != 0.0) m.bsdf_props |= LGB_FLAG_TRANSMISSION;
            if (b["reflection"].is_null() || b["reflection"].as_number() != 0.0) m.bsdf_props |= LGB_FLAG_REFLECTION;
            m.bsdf_props |= (m.ior != 1.0f && m.roughness > 0.08f) ? LGB_FLAG_GLOSSY : LGB_FLAG_SPECULAR;
            m.thin = b["thin"].is_null() ? 0u : (uint32_t)b["thin"].as_number();
        } else if (type == "conductor") {
            m.bsdf_type = LGB_BSDF_CONDUCTOR;
            m.roughness = b["roughness"].f(0.0f);
            if (!b["reflectance"].is_null()) {
                float r[3];
                for (int a = 0; a < 3; a++) r[a] = (float)b["reflectance"][a].as_number();
                conductor_from_reflectance(r, m);
            }
            if (!b["edge_tint"].is_null()) {
                // Gulbrandsen's artist-friendly mapping (JCGT 3(4) 2014), as LumenScene.cpp:425-435 applies it
                for (int a = 0; a < 3; a++) {
                    const float g = (float)b["edge_tint"][a].as_number();
                    const float r = (float)b["reflectivity"][a].as_number();
                    const float sr = std::sqrt(r);
                    const float n = g * (1.0f - r) / (1.0f + r) + (1.0f - g) * (1.0f + sr) / (1.0f - sr);
                    const float t1 = r * (n + 1.0f), t2 = n - 1.0f;
                    m.albedo[a] = n;
                    m.k[a] = std::sqrt(1.0f / (1.0f - r) * (t1 * t1 - t2 * t2));
                }
            }
            m.bsdf_props = LGB_FLAG_REFLECTION | (m.roughness > 0.08f ? LGB_FLAG_GLOSSY : LGB_FLAG_SPECULAR);
        } else if (type == "principled") {
            m.bsdf_type = LGB_BSDF_PRINCIPLED;
            m.ior = b["ior"].f(1.0f);
            m.roughness = b["roughness"].f(0.5f);
            m.diffuse_trans = b["diffuse_transmission"].f(0.0f);
            m.spec_trans = b["specular_transmission"].f(0.0f);
            m.metallic = b["metallic"].f(0.0f);
            m.specular_tint = b["specular_tint"].f(0.0f);
            m.sheen_tint = b["sheen_tint"].f(0.5f);
            m.clearcoat = b["clearcoat"].f(0.0f);
            m.clearcoat_gloss = b["clearcoat_gloss"].f(1.0f);
            m.subsurface = b["subsurface"].f(0.0f);
            m.flatness = b["flatness"].f(0.0f);
            m.sheen = b["sheen"].f(0.0f);
            m.anisotropy = b["anisotropy"].f(0.0f);
            m.thin = b["thin"].is_null() ? 0u : (uint32_t)b["thin"].as_number();
            if (m.roughness < 1.0f) m.bsdf_props |= LGB_FLAG_REFLECTION;
            if (m.spec_trans > 0.0f) m.bsdf_props |= LGB_FLAG_TRANSMISSION;
            m.bsdf_props |= m.roughness > 0.08f ? LGB_FLAG_GLOSSY : LGB_FLAG_SPECULAR;
        } else {
            // LumenScene.cpp:371-475 sets nothing for an unrecognised type ("disney" in
            // scenes/cornell_box/cornell_box_disney.json): the material keeps type 0 and no lobes, so it reflects
            // nothing and only its emission counts. The same here, with a warning.
            std::fprintf(stderr, "lgbh: bsdf type '%s' is not one Lumen's loader knows; the material reflects nothing\n",
                         type.c_str());
            m.bsdf_type = 0;
            m.bsdf_props = 0;
        }
        const Json& refs = b["refs"];
        for (size_t r = 0; r < refs.size(); r++)
            for (size_t s = 0; s < meshes.size(); s++)
                if (refs[r].as_string() == mesh_names[s]) meshes[s].material_index = (uint32_t)bi;
    }
    // camera (LumenScene.cpp:487-491)
    const Json& cam = j["camera"];
    config.cam.fov = cam["fov"].f(45.0f);
    const float zero3[3] = {0, 0, 0}, z3[3] = {0, 0, 1};
    vec3_of(cam["position"], config.cam.pos, zero3);
    vec3_of(cam["dir"], config.cam.dir, z3);
    // lights of the "lights" block (LumenScene.cpp:494-512); bounds and area lights follow in finish_lights
    const Json& jl = j["lights"];
    std::vector<lgb_light> listed;
    for (size_t i = 0; i < jl.size(); i++) {
        const Json& L = jl[i];
        lgb_light l;
        std::memset(&l, 0, sizeof(l));
        vec3_of(L["pos"], l.pos, zero3);
        vec3_of(L["dir"], l.to, zero3);
        vec3_of(L["L"], l.L, zero3);
        const std::string type = L["type"].is_null() ? std::string() : L["type"].as_string();
        if (type == "spot") l.light_flags = LGB_LIGHT_SPOT | (1u << 4) | (1u << 5);
        else if (type == "directional") l.light_flags = LGB_LIGHT_DIRECTIONAL | (1u << 5);
        else throw std::runtime_error("unknown light type '" + type + "'");
        listed.push_back(l);
    }
    finish_lights(listed);
}

// Mitsuba XML scenes as LumenScene::load_mitsuba_scene reads them (LumenScene.cpp:514-690, over
// MitsubaParser.cpp:5-147):
//  - integrator: its type selects the integrator, max_depth is the path length, enable_vm the VCM switch;
//  - sensor: fov / 2 becomes the camera's fov (LumenScene.cpp:530); its to_world matrix is copied into glm without
//    transposing (MitsubaParser.cpp:29-35), so the camera sits at the matrix's translation, and the render loop
//    rebuilds the camera from the Euler angles of its rotation (Camera.h:87-105, then update_view_matrix,
//    Camera.h:27-39): with R = Rx(a) Ry(b) Rz(c) the rotation of to_world, the camera used is T Ry(b) Rx(a) Rz(c);
//  - bsdf: twosided / mask wrappers are unwrapped to their first nested BSDF, keeping the outer id; the albedo is
//    the RGB property named "reflectance" (else another RGB property whose name contains "reflectance"), the
//    roughness sqrt(alpha), the IOR int_ior, the texture the filename of a nested texture; types map as
//    LumenScene.cpp:601-660 maps them;
//  - shape: an OBJ file (one mesh per file), its to_world transform (applied to positions and normals here; Lumen
//    passes it as the instance transform, the same geometry) and the BSDF its last reference names;
//  - emitter: sunsky becomes a directional light (L = 100 sun_color sun_scale) and sets the sky colour, which
//    the renderers then refuse as they refuse JSON directional lights. The reference iterates an unordered map of
//    properties, so whether sun_scale is applied depends on its hashing; here it always is.
// One extension: a shape's nested area emitter gives that shape an emissive copy of its material (radiance
// = the emitter's "radiance" RGB). Lumen ignores nested emitters, so no Mitsuba scene would otherwise hold an area
// light. Other emitter types are refused.
void LumenScene::load_mitsuba(const std::string& path) {
    const MtsScene sc = parse_mitsuba(read_file(path));
    const std::string root = dir_of(path);
    struct Bsdf {
        std::string name, type, texture;
        float albedo[3] = {1, 1, 1};
        float roughness = 0.0f, ior = 1.0f;
    };
    struct Shape {
        std::string file;
        int bsdf = -1;
        double m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
        bool emits = false;
        float L[3] = {0, 0, 0};
    };
    std::vector<Bsdf> bsdfs;
    std::vector<Shape> shapes;
    std::vector<lgb_light> listed;
    bool have_sensor = false;
    double cam_m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    double sensor_fov = 90.0;
    for (const MtsObject* o : sc.objects) {
        if (o->kind == "integrator") {
            config.integrator = o->plugin;
            std::transform(config.integrator.begin(), config.integrator.end(), config.integrator.begin(), ::tolower);
            if (const MtsProperty* p = o->prop("max_depth")) config.path_length = (int)p->number;
            if (const MtsProperty* p = o->prop("enable_vm")) config.enable_vm = p->boolean;
        } else if (o->kind == "sensor") {
            have_sensor = true;
            if (const MtsProperty* p = o->prop("fov")) sensor_fov = p->number;
            if (const MtsProperty* p = o->prop("to_world"))
                if (p->kind == MtsProperty::TRANSFORM) std::memcpy(cam_m, p->m, sizeof(cam_m));
        } else if (o->kind == "bsdf") {
            Bsdf b;
            b.name = o->id;
            const MtsObject* in = o;
            while ((in->plugin == "twosided" || in->plugin == "mask") && !in->anonymous.empty()) in = in->anonymous[0];
            b.type = in->plugin;
            const MtsProperty* refl = nullptr;
            for (const auto& pr : in->props)
                if (pr.second.kind == MtsProperty::COLOR && pr.first.find("reflectance") != std::string::npos)
                    if (!refl || pr.first == "reflectance") refl = &pr.second;
            if (refl)
                for (int a = 0; a < 3; a++) b.albedo[a] = (float)refl->v[a];
            if (const MtsProperty* p = in->prop("alpha")) b.roughness = (float)std::sqrt(p->number);
            if (const MtsProperty* p = in->prop("int_ior")) b.ior = (float)p->number;
            for (const auto& nc : in->named)
                if (nc.second->kind == "texture")
                    if (const MtsProperty* f = nc.second->prop("filename")) b.texture = f->text;
            bsdfs.push_back(b);
        } else if (o->kind == "shape") {
            Shape sh;
            if (const MtsProperty* p = o->prop("filename")) sh.file = p->text;
            if (const MtsProperty* p = o->prop("to_world"))
                if (p->kind == MtsProperty::TRANSFORM) std::memcpy(sh.m, p->m, sizeof(sh.m));
            for (const MtsObject* c : o->anonymous) {
                if (c->kind == "emitter") {
                    if (c->plugin != "area") throw std::runtime_error("Mitsuba: shape emitter '" + c->plugin + "' is not supported");
                    sh.emits = true;
                    if (const MtsProperty* p = c->prop("radiance"))
                        for (int a = 0; a < 3; a++) sh.L[a] = (float)p->v[a];
                    continue;
                }
                for (size_t i = 0; i < bsdfs.size(); i++)
                    if (bsdfs[i].name == c->id) sh.bsdf = (int)i;
            }
            if (sh.file.empty()) {
                std::fprintf(stderr, "lgbh: Mitsuba shape '%s' has no OBJ file and is skipped (as Lumen skips it)\n",
                             o->plugin.c_str());
                continue;
            }
            if (o->plugin != "obj") throw std::runtime_error("Mitsuba: shape type '" + o->plugin + "' is not read (OBJ only)");
            if (sh.bsdf < 0) throw std::runtime_error("Mitsuba: shape '" + sh.file + "' names no BSDF defined before it");
            shapes.push_back(sh);
        } else if (o->kind == "emitter") {
            if (o->plugin != "sunsky")
                throw std::runtime_error("Mitsuba: emitter type '" + o->plugin +
                                         "' is not read (Lumen's reader maps 'sunsky' only; area emitters go inside a shape)");
            lgb_light l;
            std::memset(&l, 0, sizeof(l));
            l.light_flags = LGB_LIGHT_DIRECTIONAL | (1u << 5);
            const MtsProperty* dir = o->prop("sun_direction");
            const MtsProperty* col = o->prop("sun_color");
            const MtsProperty* scale = o->prop("sun_scale");
            const MtsProperty* sky = o->prop("sky_color");
            for (int a = 0; a < 3; a++) {
                l.pos[a] = dir ? (float)dir->v[a] : 0.0f;
                l.L[a] = 100.0f * (col ? (float)col->v[a] : 0.0f) * (scale ? (float)scale->number : 1.0f);
                if (sky) config.sky_col[a] = (float)sky->v[a];
            }
            listed.push_back(l);
        }
    }
    // meshes (LumenScene.cpp:537-587): one per OBJ file, in shape order, transformed to world space
    for (const Shape& sh : shapes) {
        const size_t m0 = meshes.size();
        load_obj(root + sh.file);
        if (meshes.size() == m0) throw std::runtime_error("Mitsuba: " + sh.file + " has no faces");
        lgb_mesh merged = meshes[m0];
        merged.tri_count = 0;
        for (size_t k = m0; k < meshes.size(); k++) merged.tri_count += meshes[k].tri_count;
        for (uint32_t k = 0; k < 3 * merged.tri_count; k++) indices[merged.index_offset + k] = k;
        meshes.resize(m0);
        mesh_names.resize(m0);
        merged.material_index = (uint32_t)sh.bsdf;
        meshes.push_back(merged);
        mesh_names.push_back(sh.file);
        const double* M = sh.m;
        bool ident = true;
        for (int i = 0; i < 16; i++) ident = ident && M[i] == ((i % 5 == 0) ? 1.0 : 0.0);
        if (!ident) {
            // normals by the inverse transpose of the upper 3x3 (its cofactor matrix, up to a scale that the
            // normalisation removes)
            const double a = M[0], b = M[1], c = M[2], d = M[4], e = M[5], f = M[6], g = M[8], h = M[9], i = M[10];
            const double cof[9] = {e * i - f * h, f * g - d * i, d * h - e * g,
                                   c * h - b * i, a * i - c * g, b * g - a * h,
                                   b * f - c * e, c * d - a * f, a * e - b * d};
            for (size_t v = merged.vertex_offset; v < merged.vertex_offset + 3ull * merged.tri_count; v++) {
                float* p = &positions[3 * v];
                float* n = &normals[3 * v];
                const double px = p[0], py = p[1], pz = p[2], nx = n[0], ny = n[1], nz = n[2];
                for (int r = 0; r < 3; r++) p[r] = (float)(M[4 * r] * px + M[4 * r + 1] * py + M[4 * r + 2] * pz + M[4 * r + 3]);
                double q[3];
                for (int r = 0; r < 3; r++) q[r] = cof[3 * r] * nx + cof[3 * r + 1] * ny + cof[3 * r + 2] * nz;
                const double l = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
                for (int r = 0; r < 3; r++) n[r] = l > 0.0 ? (float)(q[r] / l) : 0.0f;
            }
        }
    }
    // materials (LumenScene.cpp:589-660); make_default_principled leaves every field but these at zero
    materials.assign(std::max<size_t>(bsdfs.size(), 1), default_material());
    for (size_t bi = 0; bi < bsdfs.size(); bi++) {
        const Bsdf& b = bsdfs[bi];
        lgb_material& m = materials[bi];
        if (!b.texture.empty()) {
            const std::string tex = root + b.texture;
            if (tex.size() >= 4 && tex.compare(tex.size() - 4, 4, ".pfm") == 0) {
                textures.push_back(read_pfm(tex));
                m.texture_id = (int)textures.size() - 1;
            } else {
                std::fprintf(stderr, "lgbh: texture %s skipped (only PFM textures are read)\n", tex.c_str());
            }
        }
        for (int a = 0; a < 3; a++) m.albedo[a] = b.albedo[a];
        m.roughness = b.roughness;
        if (b.type == "diffuse") {
            m.bsdf_type = LGB_BSDF_DIFFUSE;
            m.bsdf_props = LGB_FLAG_DIFFUSE | LGB_FLAG_REFLECTION;
        } else if (b.type == "roughplastic" || b.type == "roughdielectric" || b.type == "dielectric" || b.type == "plastic") {
            m.bsdf_type = LGB_BSDF_PRINCIPLED;
            m.ior = b.ior;
            if (m.roughness < 1.0f) m.bsdf_props |= LGB_FLAG_DIFFUSE | LGB_FLAG_REFLECTION;
            if (m.ior != 1.0f) m.bsdf_props |= LGB_FLAG_TRANSMISSION;
            m.bsdf_props |= m.roughness > 0.08f ? LGB_FLAG_GLOSSY : LGB_FLAG_SPECULAR;
            if (b.type == "roughdielectric" || b.type == "dielectric") {
                m.spec_trans = 1.0f;
                m.metallic = 0.0f;
            } else {  // Mitsuba's plastics mapped as LumenScene.cpp:629-635 maps them
                m.metallic = 1.0f;
                m.subsurface = 0.1f;
                m.spec_trans = 0.5f;
                m.thin = 1;
            }
        } else if (b.type == "conductor" || b.type == "roughconductor") {
            m.bsdf_type = LGB_BSDF_CONDUCTOR;
            conductor_from_reflectance(b.albedo, m);
            m.bsdf_props = LGB_FLAG_REFLECTION | (m.roughness > 0.08f ? LGB_FLAG_GLOSSY : LGB_FLAG_SPECULAR);
        } else if (b.type == "glass") {
            m.bsdf_type = LGB_BSDF_GLASS;
            m.bsdf_props = LGB_FLAG_SPECULAR | LGB_FLAG_TRANSMISSION;
            m.ior = b.ior;
        } else {
            std::fprintf(stderr, "lgbh: Mitsuba bsdf type '%s' is not one Lumen's loader maps; the material reflects "
                                 "nothing\n", b.type.c_str());
        }
    }
    // the extension: emissive copies of the materials of shapes with an area emitter
    for (size_t k = 0; k < shapes.size(); k++) {
        if (!shapes[k].emits) continue;
        lgb_material em = materials[meshes[k].material_index];
        for (int a = 0; a < 3; a++) em.emissive_factor[a] = shapes[k].L[a];
        materials.push_back(em);
        meshes[k].material_index = (uint32_t)materials.size() - 1;
    }
    // camera (LumenScene.cpp:528-534, 59-68; Camera.h:87-105, 27-39)
    if (have_sensor) {
        config.cam.use_matrix = true;
        config.cam.fov = (float)(sensor_fov / 2.0);
        const double* M = cam_m;
        double R[3][3];
        for (int c = 0; c < 3; c++) {  // rotation: the upper 3x3 with its columns normalised (scale removed)
            const double l = std::sqrt(M[c] * M[c] + M[4 + c] * M[4 + c] + M[8 + c] * M[8 + c]);
            for (int r = 0; r < 3; r++) R[r][c] = l > 0.0 ? M[4 * r + c] / l : 0.0;
        }
        const double ax = std::atan2(-R[1][2], R[2][2]);
        const double ay = std::asin(std::min(1.0, std::max(-1.0, R[0][2])));
        const double az = std::atan2(-R[0][1], R[0][0]);
        auto rot = [](int axis, double t, double out[3][3]) {
            const double c = std::cos(t), s = std::sin(t);
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++) out[r][q] = r == q ? 1.0 : 0.0;
            const int u = (axis + 1) % 3, v = (axis + 2) % 3;
            out[u][u] = c; out[u][v] = -s; out[v][u] = s; out[v][v] = c;
        };
        auto mul = [](const double a[3][3], const double b[3][3], double out[3][3]) {
            double t[3][3];
            for (int r = 0; r < 3; r++)
                for (int q = 0; q < 3; q++) t[r][q] = a[r][0] * b[0][q] + a[r][1] * b[1][q] + a[r][2] * b[2][q];
            std::memcpy(out, t, sizeof(t));
        };
        double Ry[3][3], Rx[3][3], Rz[3][3], C[3][3];
        rot(1, ay, Ry);
        rot(0, ax, Rx);
        rot(2, az, Rz);
        mul(Ry, Rx, C);
        mul(C, Rz, C);
        float* out = config.cam.cam_matrix;  // column-major
        for (int c = 0; c < 3; c++) {
            for (int r = 0; r < 3; r++) out[4 * c + r] = (float)C[r][c];
            out[4 * c + 3] = 0.0f;
        }
        out[12] = (float)M[3];
        out[13] = (float)M[7];
        out[14] = (float)M[11];
        out[15] = 1.0f;
        for (int a = 0; a < 3; a++) config.cam.pos[a] = out[12 + a];
    }
    finish_lights(listed);
}

// Scene bounds, then the light list as LumenScene::load_scene builds it (LumenScene.cpp:70-113): every mesh with
// an emissive material becomes an area light, then the listed lights follow with the scene's centre and radius.
void LumenScene::finish_lights(const std::vector<lgb_light>& listed) {
    // scene bounds (LumenScene.cpp:732-751): from the meshes' vertex bounds; a degenerate box becomes [-1, 1]^3
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < positions.size(); i += 3)
        for (int a = 0; a < 3; a++) { lo[a] = std::min(lo[a], positions[i + a]); hi[a] = std::max(hi[a], positions[i + a]); }
    if (!(lo[0] < hi[0] && lo[1] < hi[1] && lo[2] < hi[2])) {
        for (int a = 0; a < 3; a++) { lo[a] = -1.0f; hi[a] = 1.0f; }
    }
    float d2 = 0.0f;
    for (int a = 0; a < 3; a++) { bbox_min[a] = lo[a]; bbox_max[a] = hi[a]; d2 += (hi[a] - lo[a]) * (hi[a] - lo[a]); }
    radius = std::sqrt(d2) * 0.5f;
    total_light_triangle_cnt = 0;
    for (size_t s = 0; s < meshes.size(); s++) {
        const lgb_material& mat = materials[meshes[s].material_index];
        const float* e = mat.emissive_factor;
        if (e[0] > 0 || e[1] > 0 || e[2] > 0) {
            lgb_light l;
            std::memset(&l, 0, sizeof(l));
            for (int i = 0; i < 4; i++) l.world_matrix[5 * i] = 1.0f;
            l.num_triangles = meshes[s].tri_count;
            l.prim_mesh_idx = (uint32_t)s;
            l.light_flags = LGB_LIGHT_AREA | (1u << 4);
            for (int a = 0; a < 3; a++) l.L[a] = e[a];
            lights.push_back(l);
            total_light_triangle_cnt += l.num_triangles;
            for (uint32_t t = 0; t < meshes[s].tri_count; t++) {
                const uint32_t base = meshes[s].index_offset + 3 * t;
                const float* p0 = &positions[3 * (size_t)(indices[base] + meshes[s].vertex_offset)];
                const float* p1 = &positions[3 * (size_t)(indices[base + 1] + meshes[s].vertex_offset)];
                const float* p2 = &positions[3 * (size_t)(indices[base + 2] + meshes[s].vertex_offset)];
                const float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                const float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                const float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
                total_light_area += 0.5f * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
            }
        }
    }
    for (size_t i = 0; i < listed.size(); i++) {
        lgb_light l = listed[i];
        std::memset(l.world_matrix, 0, sizeof(l.world_matrix));
        for (int k = 0; k < 4; k++) l.world_matrix[5 * k] = 1.0f;
        l.world_radius = radius;
        for (int a = 0; a < 3; a++) l.world_center[a] = 0.5f * (bbox_max[a] + bbox_min[a]);
        // the index into the listed lights, as LumenScene.cpp:104-106 records it
        if ((l.light_flags & 7u) == LGB_LIGHT_DIRECTIONAL) dir_light_idx = (uint32_t)i;
        total_light_triangle_cnt++;
        lights.push_back(l);
    }
}

std::vector<lgb_texture> LumenScene::texture_views() const {
    std::vector<lgb_texture> v;
    for (const TextureData& t : textures) v.push_back({t.width, t.height, t.rgba.data()});
    return v;
}

lgb_scene_desc LumenScene::desc() const {
    tex_views_ = texture_views();
    lgb_scene_desc d;
    std::memset(&d, 0, sizeof(d));
    d.positions = positions.data();
    d.normals = normals.data();
    d.uvs = uvs.data();
    d.num_vertices = (uint32_t)(positions.size() / 3);
    d.indices = indices.data();
    d.num_indices = (uint32_t)indices.size();
    d.meshes = meshes.data();
    d.num_meshes = (uint32_t)meshes.size();
    d.materials = materials.data();
    d.num_materials = (uint32_t)materials.size();
    d.lights = lights.empty() ? nullptr : lights.data();
    d.num_lights = (uint32_t)lights.size();
    d.textures = tex_views_.empty() ? nullptr : tex_views_.data();
    d.num_textures = (uint32_t)tex_views_.size();
    return d;
}

TextureData read_pfm(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::string magic;
    uint32_t w = 0, h = 0;
    float scale = 0.0f;
    f >> magic >> w >> h >> scale;
    f.get();
    if ((magic != "PF" && magic != "Pf") || w == 0 || h == 0) throw std::runtime_error("not a PFM file: " + path);
    const int ch = magic == "PF" ? 3 : 1;
    std::vector<float> raw((size_t)w * h * ch);
    f.read(reinterpret_cast<char*>(raw.data()), raw.size() * 4);
    if (!f) throw std::runtime_error("truncated PFM file: " + path);
    const bool little = scale < 0.0f;
    const uint16_t probe = 1;
    const bool host_little = *reinterpret_cast<const uint8_t*>(&probe) == 1;
    if (little != host_little)
        for (float& x : raw) {
            uint8_t* b = reinterpret_cast<uint8_t*>(&x);
            std::swap(b[0], b[3]);
            std::swap(b[1], b[2]);
        }
    TextureData t;
    t.width = w;
    t.height = h;
    t.rgba.resize((size_t)w * h * 4);
    for (uint32_t y = 0; y < h; y++)  // PFM rows run bottom-up
        for (uint32_t x = 0; x < w; x++) {
            const float* src = &raw[((size_t)(h - 1 - y) * w + x) * ch];
            float* dst = &t.rgba[((size_t)y * w + x) * 4];
            for (int a = 0; a < 3; a++) dst[a] = src[ch == 3 ? a : 0];
            dst[3] = 1.0f;
        }
    return t;
}

void write_pfm(const std::string& path, const float* rgba, uint32_t width, uint32_t height) {
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + path);
    const uint16_t probe = 1;
    const bool host_little = *reinterpret_cast<const uint8_t*>(&probe) == 1;
    f << "PF\n" << width << " " << height << "\n" << (host_little ? "-1.0" : "1.0") << "\n";
    std::vector<float> row((size_t)width * 3);
    for (uint32_t y = 0; y < height; y++) {
        const uint32_t src_y = height - 1 - y;
        for (uint32_t x = 0; x < width; x++)
            for (int a = 0; a < 3; a++) row[(size_t)x * 3 + a] = rgba[((size_t)src_y * width + x) * 4 + a];
        f.write(reinterpret_cast<const char*>(row.data()), row.size() * 4);
    }
}

namespace {
// Little-endian byte writers for the OpenEXR header and scanline blocks.
void put_u32(std::string& b, uint32_t v) { for (int k = 0; k < 4; k++) b.push_back((char)((v >> (8 * k)) & 0xffu)); }
void put_u64(std::string& b, uint64_t v) { for (int k = 0; k < 8; k++) b.push_back((char)((v >> (8 * k)) & 0xffu)); }
void put_f32(std::string& b, float f) {
    uint32_t v;
    std::memcpy(&v, &f, 4);
    put_u32(b, v);
}
void put_attr(std::string& b, const char* name, const char* type, const std::string& value) {
    b.append(name);
    b.push_back('\0');
    b.append(type);
    b.push_back('\0');
    put_u32(b, (uint32_t)value.size());
    b.append(value);
}
}  // namespace

// OpenEXR 2.0, single-part scanline image, no compression, channels B, G, R as 32-bit floats (channel records
// in alphabetical order, as the format requires), one scanline per block, the offset table after the header.
// Rows run top-down, as in the film. Written from the published file layout; stands in for the tinyexr call of
// ImageUtils.cpp:22-89.
void write_exr(const std::string& path, const float* rgba, uint32_t width, uint32_t height) {
    if (width == 0 || height == 0 || width > 0x7fffffffu || height > 0x7fffffffu)
        throw std::runtime_error("bad image size for " + path);
    std::string b;
    put_u32(b, 20000630u);  // magic 0x762f3101
    put_u32(b, 2u);         // version 2, single-part scanline
    std::string ch;
    for (const char* c : {"B", "G", "R"}) {
        ch.append(c);
        ch.push_back('\0');
        put_u32(ch, 2u);            // pixel type FLOAT
        ch.append(4, '\0');         // pLinear = 0, three reserved bytes
        put_u32(ch, 1u);            // x sampling
        put_u32(ch, 1u);            // y sampling
    }
    ch.push_back('\0');
    put_attr(b, "channels", "chlist", ch);
    put_attr(b, "compression", "compression", std::string(1, '\0'));
    std::string box;
    put_u32(box, 0u);
    put_u32(box, 0u);
    put_u32(box, width - 1u);
    put_u32(box, height - 1u);
    put_attr(b, "dataWindow", "box2i", box);
    put_attr(b, "displayWindow", "box2i", box);
    put_attr(b, "lineOrder", "lineOrder", std::string(1, '\0'));  // increasing y
    std::string one;
    put_f32(one, 1.0f);
    put_attr(b, "pixelAspectRatio", "float", one);
    std::string center;
    put_f32(center, 0.0f);
    put_f32(center, 0.0f);
    put_attr(b, "screenWindowCenter", "v2f", center);
    put_attr(b, "screenWindowWidth", "float", one);
    b.push_back('\0');  // end of header
    const uint64_t row_bytes = 3ull * 4ull * width;
    const uint64_t block_bytes = 8ull + row_bytes;
    const uint64_t first = b.size() + 8ull * height;
    for (uint32_t y = 0; y < height; y++) put_u64(b, first + (uint64_t)y * block_bytes);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + path);
    f.write(b.data(), (std::streamsize)b.size());
    std::string row;
    row.reserve((size_t)block_bytes);
    for (uint32_t y = 0; y < height; y++) {
        row.clear();
        put_u32(row, y);
        put_u32(row, (uint32_t)row_bytes);
        for (int c : {2, 1, 0})  // B, G, R planes of the row
            for (uint32_t x = 0; x < width; x++) put_f32(row, rgba[((size_t)y * width + x) * 4 + c]);
        f.write(row.data(), (std::streamsize)row.size());
    }
    if (!f) throw std::runtime_error("write failed: " + path);
}

// ".exr" writes OpenEXR, anything else PFM.
void write_image(const std::string& path, const float* rgba, uint32_t width, uint32_t height) {
    const bool exr = path.size() >= 4 && (path.compare(path.size() - 4, 4, ".exr") == 0 ||
                                          path.compare(path.size() - 4, 4, ".EXR") == 0);
    if (exr) write_exr(path, rgba, width, height);
    else write_pfm(path, rgba, width, height);
}

}  // namespace lgbh
