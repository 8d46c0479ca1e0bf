// Mitsuba XML scene files, the subset Lumen reads (src/Framework/MitsubaParser.cpp:5-147, on top of the vendored
// tinyparser-mitsuba 0.1): a small XML reader and the Mitsuba object model of integrators, sensors, BSDFs,
// shapes and emitters with their typed properties. Our own code for the same file format.
#pragma once
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace lgbh {

// One XML element: tag, attributes in document order, child elements (text content is ignored: Mitsuba scene
// files carry everything in attributes).
struct XmlNode {
    std::string tag;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XmlNode> children;
    const std::string* attr(const char* name) const;
};
// Parses a whole document and returns its root element. Skips the declaration, comments, processing
// instructions and DOCTYPE; decodes the five predefined entities and numeric character references in attribute
// values. Throws std::runtime_error with the byte offset of the first syntax error.
XmlNode parse_xml(const std::string& text);

struct MtsProperty {
    enum Kind { INTEGER, FLOAT, BOOLEAN, STRING, COLOR, VECTOR, TRANSFORM } kind = FLOAT;
    double number = 0.0;    // INTEGER, FLOAT
    bool boolean = false;   // BOOLEAN
    std::string text;       // STRING
    double v[3] = {0, 0, 0};  // COLOR (r, g, b), VECTOR / point (x, y, z)
    double m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // TRANSFORM, row-major
};

struct MtsObject {
    std::string kind;    // element name: integrator, sensor, bsdf, shape, emitter, texture, ...
    std::string plugin;  // the "type" attribute
    std::string id;
    std::vector<std::pair<std::string, MtsProperty>> props;         // in document order
    std::vector<const MtsObject*> anonymous;                         // child objects and references without a name
    std::vector<std::pair<std::string, const MtsObject*>> named;     // child objects and references with a name
    const MtsProperty* prop(const std::string& name) const;         // last property of that name, or null
};

struct MtsScene {
    int version_major = 0;
    std::vector<const MtsObject*> objects;  // the scene's anonymous children, in document order
    std::vector<std::unique_ptr<MtsObject>> storage;
};

// Loads a Mitsuba scene file. Version-0 files have their camelCase property and child names lowered to
// snake_case ("maxDepth" -> "max_depth", "enableVM" -> "enable_vm", "toWorld" -> "to_world"), the names
// MitsubaParser.cpp:15-18,26,56,62 look for. <ref id> resolves to an object defined earlier in the file.
// <transform> composes its translate / scale / rotate / lookat / matrix children, each applied after the
// ones before it. Throws std::runtime_error on malformed input.
MtsScene parse_mitsuba(const std::string& text);

// camelCase -> snake_case as version-0 scene names need: '_' before an upper-case letter that follows a
// lower-case one, then everything lowered.
std::string mitsuba_snake_case(const std::string& name);

}  // namespace lgbh
