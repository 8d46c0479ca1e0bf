// Mitsuba XML scene files: XML reader and object model. See mitsuba_xml.h.
#include "mitsuba_xml.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>

namespace lgbh {

const std::string* XmlNode::attr(const char* name) const {
    for (const auto& a : attrs)
        if (a.first == name) return &a.second;
    return nullptr;
}

namespace {

class XmlReader {
  public:
    explicit XmlReader(const std::string& s) : s_(s) {}

    XmlNode document() {
        skip_misc();
        if (i_ >= s_.size() || s_[i_] != '<') fail("no root element");
        XmlNode root = element(0);
        skip_misc();
        return root;
    }

  private:
    const std::string& s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const std::string& what) const {
        throw std::runtime_error("XML: " + what + " at byte " + std::to_string(i_));
    }
    bool at(const char* p) const { return s_.compare(i_, std::strlen(p), p) == 0; }
    void skip_ws() {
        while (i_ < s_.size() && std::isspace((unsigned char)s_[i_])) i_++;
    }
    void skip_to(const char* end) {
        const size_t e = s_.find(end, i_);
        if (e == std::string::npos) fail(std::string("missing '") + end + "'");
        i_ = e + std::strlen(end);
    }
    // Whitespace, comments, processing instructions and DOCTYPE between elements.
    void skip_misc() {
        for (;;) {
            skip_ws();
            if (at("<!--")) skip_to("-->");
            else if (at("<?")) skip_to("?>");
            else if (at("<!DOCTYPE") || at("<!doctype")) skip_to(">");
            else return;
        }
    }
    std::string name() {
        const size_t b = i_;
        while (i_ < s_.size() && (std::isalnum((unsigned char)s_[i_]) || std::strchr("_:-.", s_[i_]) != nullptr)) i_++;
        if (b == i_) fail("expected a name");
        return s_.substr(b, i_ - b);
    }
    static void put_utf8(std::string& out, unsigned long c) {
        if (c < 0x80) {
            out.push_back((char)c);
        } else if (c < 0x800) {
            out.push_back((char)(0xC0 | (c >> 6)));
            out.push_back((char)(0x80 | (c & 0x3F)));
        } else if (c < 0x10000) {
            out.push_back((char)(0xE0 | (c >> 12)));
            out.push_back((char)(0x80 | ((c >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (c & 0x3F)));
        } else {
            out.push_back((char)(0xF0 | (c >> 18)));
            out.push_back((char)(0x80 | ((c >> 12) & 0x3F)));
            out.push_back((char)(0x80 | ((c >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (c & 0x3F)));
        }
    }
    std::string decode(const std::string& raw) const {
        std::string out;
        for (size_t k = 0; k < raw.size(); k++) {
            if (raw[k] != '&') {
                out.push_back(raw[k]);
                continue;
            }
            const size_t e = raw.find(';', k);
            if (e == std::string::npos) fail("unterminated entity in an attribute value");
            const std::string ent = raw.substr(k + 1, e - k - 1);
            if (ent == "amp") out.push_back('&');
            else if (ent == "lt") out.push_back('<');
            else if (ent == "gt") out.push_back('>');
            else if (ent == "quot") out.push_back('"');
            else if (ent == "apos") out.push_back('\'');
            else if (ent.size() > 1 && ent[0] == '#') {
                const bool hex = ent[1] == 'x' || ent[1] == 'X';
                char* end = nullptr;
                const unsigned long c = std::strtoul(ent.c_str() + (hex ? 2 : 1), &end, hex ? 16 : 10);
                if (!end || *end != '\0' || c > 0x10FFFF) fail("bad character reference &" + ent + ";");
                put_utf8(out, c);
            } else {
                fail("unknown entity &" + ent + ";");
            }
            k = e;
        }
        return out;
    }
    XmlNode element(int depth) {
        if (depth > 256) fail("elements nested too deeply");
        i_++;  // '<'
        XmlNode n;
        n.tag = name();
        for (;;) {
            skip_ws();
            if (at("/>")) {
                i_ += 2;
                return n;
            }
            if (i_ < s_.size() && s_[i_] == '>') {
                i_++;
                break;
            }
            std::string an = name();
            skip_ws();
            if (i_ >= s_.size() || s_[i_] != '=') fail("expected '=' after attribute " + an);
            i_++;
            skip_ws();
            if (i_ >= s_.size() || (s_[i_] != '"' && s_[i_] != '\'')) fail("expected a quoted value for " + an);
            const char q = s_[i_];
            const size_t e = s_.find(q, i_ + 1);
            if (e == std::string::npos) fail("unterminated value of attribute " + an);
            n.attrs.emplace_back(an, decode(s_.substr(i_ + 1, e - i_ - 1)));
            i_ = e + 1;
        }
        for (;;) {
            while (i_ < s_.size() && s_[i_] != '<') i_++;  // character data is not used
            if (i_ >= s_.size()) fail("element <" + n.tag + "> is not closed");
            if (at("<!--")) skip_to("-->");
            else if (at("<![CDATA[")) skip_to("]]>");
            else if (at("<?")) skip_to("?>");
            else if (at("</")) {
                i_ += 2;
                const std::string t = name();
                if (t != n.tag) fail("</" + t + "> closes <" + n.tag + ">");
                skip_ws();
                if (i_ >= s_.size() || s_[i_] != '>') fail("expected '>'");
                i_++;
                return n;
            } else {
                n.children.push_back(element(depth + 1));
            }
        }
    }
};

bool is_object_tag(const std::string& t) {
    static const char* const kinds[] = {"integrator", "sensor", "bsdf", "shape", "emitter", "texture", "sampler",
                                        "film", "rfilter", "medium", "phase", "subsurface", "volume"};
    for (const char* k : kinds)
        if (t == k) return true;
    return false;
}

// Row-major 4x4 products and the elementary transforms of a Mitsuba <transform>.
void mat_mul(const double a[16], const double b[16], double out[16]) {
    double r[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double acc = 0.0;
            for (int k = 0; k < 4; k++) acc += a[4 * i + k] * b[4 * k + j];
            r[4 * i + j] = acc;
        }
    std::memcpy(out, r, sizeof(r));
}
void identity(double m[16]) {
    for (int i = 0; i < 16; i++) m[i] = (i % 5 == 0) ? 1.0 : 0.0;
}

class Builder {
  public:
    explicit Builder(MtsScene& sc) : sc_(sc) {}

    void scene(const XmlNode& root) {
        if (root.tag != "scene") throw std::runtime_error("Mitsuba: the root element is <" + root.tag + ">, not <scene>");
        sc_.version_major = 0;  // a file without a version is read as 0.x
        if (const std::string* v = root.attr("version")) sc_.version_major = std::atoi(v->c_str());
        snake_ = sc_.version_major == 0;
        for (const XmlNode& c : root.children) {
            if (is_object_tag(c.tag)) {
                const MtsObject* o = object(c);
                if (!c.attr("name")) sc_.objects.push_back(o);
            } else if (c.tag == "ref") {
                sc_.objects.push_back(resolve(c));
            } else {
                throw std::runtime_error("Mitsuba: unsupported element <" + c.tag + "> in <scene>");
            }
        }
    }

  private:
    MtsScene& sc_;
    bool snake_ = true;
    std::map<std::string, const MtsObject*> ids_;

    std::string prop_name(const XmlNode& e) const {
        const std::string* n = e.attr("name");
        if (!n) throw std::runtime_error("Mitsuba: <" + e.tag + "> has no name");
        return snake_ ? mitsuba_snake_case(*n) : *n;
    }
    static std::vector<double> numbers(const std::string& text, const std::string& what) {
        std::vector<double> out;
        const char* p = text.c_str();
        for (;;) {
            while (*p && (std::isspace((unsigned char)*p) || *p == ',')) p++;
            if (!*p) break;
            char* end = nullptr;
            const double v = std::strtod(p, &end);
            if (end == p) throw std::runtime_error("Mitsuba: cannot read the numbers of " + what + " from '" + text + "'");
            out.push_back(v);
            p = end;
        }
        return out;
    }
    static const std::string& need(const XmlNode& e, const char* a) {
        const std::string* v = e.attr(a);
        if (!v) throw std::runtime_error("Mitsuba: <" + e.tag + "> has no '" + a + "' attribute");
        return *v;
    }
    static void vec3(const XmlNode& e, const std::string& what, double out[3]) {
        if (const std::string* v = e.attr("value")) {
            const std::vector<double> n = numbers(*v, what);
            if (n.size() == 1) { out[0] = out[1] = out[2] = n[0]; return; }
            if (n.size() != 3) throw std::runtime_error("Mitsuba: " + what + " needs 1 or 3 values");
            for (int k = 0; k < 3; k++) out[k] = n[k];
            return;
        }
        const char* xyz[3] = {"x", "y", "z"};
        const char* rgb[3] = {"r", "g", "b"};
        for (int k = 0; k < 3; k++) {
            const std::string* s = e.attr(xyz[k]);
            if (!s) s = e.attr(rgb[k]);
            out[k] = s ? numbers(*s, what).at(0) : 0.0;
        }
    }
    static void transform_step(const XmlNode& t, double m[16]) {
        identity(m);
        if (t.tag == "translate") {
            double d[3];
            vec3(t, "translate", d);
            m[3] = d[0]; m[7] = d[1]; m[11] = d[2];
        } else if (t.tag == "scale") {
            double d[3] = {1, 1, 1};
            if (t.attr("value")) vec3(t, "scale", d);
            else for (int k = 0; k < 3; k++) { const char* a[3] = {"x", "y", "z"}; if (const std::string* s = t.attr(a[k])) d[k] = numbers(*s, "scale").at(0); }
            m[0] = d[0]; m[5] = d[1]; m[10] = d[2];
        } else if (t.tag == "rotate") {
            // rotation by `angle` degrees about the axis (x, y, z), right-handed (Rodrigues' formula)
            double ax[3];
            vec3(t, "rotate axis", ax);
            const double ang = numbers(need(t, "angle"), "rotate angle").at(0) * (3.14159265358979323846 / 180.0);
            const double l = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
            if (!(l > 0.0)) throw std::runtime_error("Mitsuba: rotate needs a non-zero axis");
            const double x = ax[0] / l, y = ax[1] / l, z = ax[2] / l, c = std::cos(ang), s = std::sin(ang), k = 1.0 - c;
            const double r[9] = {c + x * x * k, x * y * k - z * s, x * z * k + y * s,
                                 y * x * k + z * s, c + y * y * k, y * z * k - x * s,
                                 z * x * k - y * s, z * y * k + x * s, c + z * z * k};
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++) m[4 * i + j] = r[3 * i + j];
        } else if (t.tag == "lookat" || t.tag == "lookAt") {
            // camera-to-world of a camera at `origin` looking at `target`: columns left, up, forward, origin
            const std::vector<double> o = numbers(need(t, "origin"), "lookat origin");
            const std::vector<double> g = numbers(need(t, "target"), "lookat target");
            std::vector<double> up = {0, 1, 0};
            if (const std::string* u = t.attr("up")) up = numbers(*u, "lookat up");
            if (o.size() != 3 || g.size() != 3 || up.size() != 3) throw std::runtime_error("Mitsuba: lookat needs 3-vectors");
            auto norm = [](double v[3]) {
                const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                if (!(l > 0.0)) throw std::runtime_error("Mitsuba: degenerate lookat");
                for (int k = 0; k < 3; k++) v[k] /= l;
            };
            auto cross = [](const double a[3], const double b[3], double r[3]) {
                r[0] = a[1] * b[2] - a[2] * b[1]; r[1] = a[2] * b[0] - a[0] * b[2]; r[2] = a[0] * b[1] - a[1] * b[0];
            };
            double f[3] = {g[0] - o[0], g[1] - o[1], g[2] - o[2]}, u[3] = {up[0], up[1], up[2]}, left[3], nu[3];
            norm(f);
            cross(u, f, left);
            norm(left);
            cross(f, left, nu);
            norm(nu);
            for (int i = 0; i < 3; i++) {
                m[4 * i + 0] = left[i]; m[4 * i + 1] = nu[i]; m[4 * i + 2] = f[i]; m[4 * i + 3] = o[i];
            }
        } else if (t.tag == "matrix") {
            const std::vector<double> n = numbers(need(t, "value"), "matrix");
            if (n.size() == 9) {
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) m[4 * i + j] = n[3 * i + j];
            } else if (n.size() == 12 || n.size() == 16) {
                for (size_t k = 0; k < n.size(); k++) m[k] = n[k];
            } else {
                throw std::runtime_error("Mitsuba: a matrix needs 9, 12 or 16 values");
            }
        } else {
            throw std::runtime_error("Mitsuba: unsupported transform element <" + t.tag + ">");
        }
    }
    // Returns false for property elements this reader skips (spectra, blackbody emitters).
    bool property(const XmlNode& e, MtsProperty& p) const {
        const std::string& t = e.tag;
        if (t == "integer" || t == "float") {
            p.kind = t == "integer" ? MtsProperty::INTEGER : MtsProperty::FLOAT;
            p.number = numbers(need(e, "value"), t).at(0);
        } else if (t == "boolean") {
            const std::string& v = need(e, "value");
            if (v != "true" && v != "false") throw std::runtime_error("Mitsuba: boolean value '" + v + "'");
            p.kind = MtsProperty::BOOLEAN;
            p.boolean = v == "true";
        } else if (t == "string") {
            p.kind = MtsProperty::STRING;
            p.text = need(e, "value");
        } else if (t == "rgb") {
            p.kind = MtsProperty::COLOR;
            vec3(e, "rgb", p.v);
        } else if (t == "vector" || t == "point") {
            p.kind = MtsProperty::VECTOR;
            vec3(e, t, p.v);
        } else if (t == "transform") {
            p.kind = MtsProperty::TRANSFORM;
            identity(p.m);
            for (const XmlNode& c : e.children) {
                double step[16];
                transform_step(c, step);
                mat_mul(step, p.m, p.m);  // each step is applied after the ones before it
            }
        } else if (t == "spectrum" || t == "blackbody") {
            return false;
        } else {
            throw std::runtime_error("Mitsuba: unsupported element <" + t + ">");
        }
        return true;
    }
    const MtsObject* resolve(const XmlNode& r) const {
        const std::string& id = need(r, "id");
        const auto it = ids_.find(id);
        if (it == ids_.end()) throw std::runtime_error("Mitsuba: <ref id=\"" + id + "\"> names no object defined before it");
        return it->second;
    }
    const MtsObject* object(const XmlNode& e) {
        sc_.storage.push_back(std::make_unique<MtsObject>());
        MtsObject* o = sc_.storage.back().get();
        o->kind = e.tag;
        if (const std::string* t = e.attr("type")) o->plugin = *t;
        if (const std::string* id = e.attr("id")) o->id = *id;
        for (const XmlNode& c : e.children) {
            const MtsObject* child = nullptr;
            if (is_object_tag(c.tag)) child = object(c);
            else if (c.tag == "ref") child = resolve(c);
            if (child) {
                if (c.attr("name")) o->named.emplace_back(prop_name(c), child);
                else o->anonymous.push_back(child);
                continue;
            }
            MtsProperty p;
            if (!property(c, p)) continue;
            const std::string n = prop_name(c);
            bool replaced = false;  // one value per name: a later definition replaces an earlier one
            for (auto& q : o->props)
                if (q.first == n) { q.second = p; replaced = true; }
            if (!replaced) o->props.emplace_back(n, p);
        }
        if (!o->id.empty()) ids_[o->id] = o;
        return o;
    }
};

}  // namespace

const MtsProperty* MtsObject::prop(const std::string& name) const {
    const MtsProperty* r = nullptr;
    for (const auto& p : props)
        if (p.first == name) r = &p.second;
    return r;
}

std::string mitsuba_snake_case(const std::string& name) {
    std::string out;
    for (size_t k = 0; k < name.size(); k++) {
        const char c = name[k];
        if (k > 0 && std::isupper((unsigned char)c) && std::islower((unsigned char)name[k - 1])) out.push_back('_');
        out.push_back((char)std::tolower((unsigned char)c));
    }
    return out;
}

XmlNode parse_xml(const std::string& text) { return XmlReader(text).document(); }

MtsScene parse_mitsuba(const std::string& text) {
    const XmlNode root = parse_xml(text);
    MtsScene sc;
    Builder(sc).scene(root);
    return sc;
}

}  // namespace lgbh
