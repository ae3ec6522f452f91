// scene_file.cpp — WalkRay's scene files read into a wr_scene_desc, host only
// (wr_scene_file_load / wr_scene_file_get / wr_scene_file_free).
//
// Follows Config::load (config.cpp:432-575), Config::generateSceneObject
// (config.cpp:21-430) and Mesh::loadShape (mesh.cpp:5-130), including the
// reference's own behaviour where it is surprising:
//  * a single <Object>'s mesh is unitized in place (loadShape's default
//    normalize = true, mesh.h:34): centred on its bounding box and scaled by
//    2 / (largest extent), then placed by the object's <transform>;
//  * a <GroupObject>'s shapes are scaled by the matrix Mesh::unitize returns
//    (mesh.cpp:144-158); that matrix is built with nvMatrix's 16-argument
//    constructor, which stores its arguments column by column, so the
//    translation lands in the w row and the shapes are scaled but not
//    centred; every object of the group then takes the group's <transform>
//    (copyMesh after the object's own transform, config.cpp:52-57); an object
//    naming no group of the file gets the whole file, unitized, and its own
//    <transform> (generateSceneObject with no shape);
//  * a .shp file stores a count n, then n floats of vertex data that are read
//    into n vertices, then a count m and m unsigned of face data read into m
//    faces (mesh.cpp:20-25): the vertices and faces past the first n / 3 and
//    m / 3 are zero;
//  * an .obj face keeps its first three vertices; v, v/vt, v/vt/vn and v//vn
//    forms are read (mesh.cpp:57-90); vertex normals are not used by this
//    renderer (face normals only) and are skipped;
//  * world positions are transform * (v, 1) with nvMatrix's operation order
//    (nvMatrix.h:424-433), in FP32 without contraction, the x, y, z of the
//    result; the <transform> text is row-major (readMatrix, config.cpp:610-619).
// Values are read a little more leniently than sscanf in the reference
// (whitespace around numbers and names is accepted); everything the reference
// reads is read to the same numbers.  Not supported (an error names them):
// BumpMapping materials, <motion> (the reference renders one random instant
// per object, chosen at load time), and subsurface grid volumes.
#include <sys/stat.h>

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/walkray.h"

namespace {

// ---------------------------------------------------------------------------
// a small XML reader: elements, attributes, text, comments, declarations
// ---------------------------------------------------------------------------
struct XNode {
    std::string tag;
    std::map<std::string, std::string> attrs;
    std::string text;  // the first run of character data (rapidxml's value())
    bool has_text = false;
    std::vector<std::unique_ptr<XNode>> kids;

    const XNode* first(const char* t) const {
        for (auto& k : kids)
            if (k->tag == t) return k.get();
        return nullptr;
    }
    const char* value() const { return text.c_str(); }
    const std::string* attr(const char* a) const {
        auto it = attrs.find(a);
        return it == attrs.end() ? nullptr : &it->second;
    }
};

struct XmlParser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit XmlParser(const std::string& src) : s(src) {}

    static std::string decode(const std::string& in) {
        std::string out;
        for (size_t k = 0; k < in.size(); k++) {
            if (in[k] != '&') {
                out += in[k];
                continue;
            }
            const size_t e = in.find(';', k);
            if (e == std::string::npos) {
                out += in[k];
                continue;
            }
            const std::string ent = in.substr(k + 1, e - k - 1);
            if (ent == "lt") out += '<';
            else if (ent == "gt") out += '>';
            else if (ent == "amp") out += '&';
            else if (ent == "quot") out += '"';
            else if (ent == "apos") out += '\'';
            else out += in.substr(k, e - k + 1);
            k = e;
        }
        return out;
    }
    void skip_ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    bool starts(const char* p) const { return s.compare(i, strlen(p), p) == 0; }
    // skips a comment, <?...?> or <!...> at position i; true if one was there
    bool skip_misc() {
        if (starts("<!--")) {
            const size_t e = s.find("-->", i + 4);
            i = e == std::string::npos ? s.size() : e + 3;
            return true;
        }
        if (starts("<?")) {
            const size_t e = s.find("?>", i + 2);
            i = e == std::string::npos ? s.size() : e + 2;
            return true;
        }
        if (starts("<!")) {
            const size_t e = s.find('>', i + 2);
            i = e == std::string::npos ? s.size() : e + 1;
            return true;
        }
        return false;
    }
    std::string name() {
        const size_t b = i;
        while (i < s.size() && !std::isspace((unsigned char)s[i]) && s[i] != '>' && s[i] != '/' && s[i] != '=')
            i++;
        return s.substr(b, i - b);
    }
    // the element starting at s[i] == '<'
    std::unique_ptr<XNode> element(int depth) {
        if (depth > 256) {
            err = "XML nesting too deep";
            return nullptr;
        }
        auto n = std::make_unique<XNode>();
        i++;  // '<'
        n->tag = name();
        if (n->tag.empty()) {
            err = "malformed XML tag";
            return nullptr;
        }
        for (;;) {
            skip_ws();
            if (i >= s.size()) {
                err = "unterminated XML tag <" + n->tag + ">";
                return nullptr;
            }
            if (starts("/>")) {
                i += 2;
                return n;
            }
            if (s[i] == '>') {
                i++;
                break;
            }
            const std::string a = name();
            skip_ws();
            if (a.empty() || i >= s.size() || s[i] != '=') {
                err = "malformed attribute in <" + n->tag + ">";
                return nullptr;
            }
            i++;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) {
                err = "unquoted attribute in <" + n->tag + ">";
                return nullptr;
            }
            const char q = s[i++];
            const size_t e = s.find(q, i);
            if (e == std::string::npos) {
                err = "unterminated attribute in <" + n->tag + ">";
                return nullptr;
            }
            n->attrs[a] = decode(s.substr(i, e - i));
            i = e + 1;
        }
        for (;;) {  // content
            if (i >= s.size()) {
                err = "missing </" + n->tag + ">";
                return nullptr;
            }
            if (starts("</")) {
                i += 2;
                const std::string t = name();
                skip_ws();
                if (t != n->tag || i >= s.size() || s[i] != '>') {
                    err = "mismatched </" + t + "> for <" + n->tag + ">";
                    return nullptr;
                }
                i++;
                return n;
            }
            if (skip_misc()) continue;
            if (s[i] == '<') {
                auto k = element(depth + 1);
                if (!k) return nullptr;
                n->kids.push_back(std::move(k));
                continue;
            }
            const size_t e = s.find('<', i);
            const std::string data = s.substr(i, (e == std::string::npos ? s.size() : e) - i);
            if (!n->has_text) {
                bool blank = true;
                for (char c : data) blank = blank && std::isspace((unsigned char)c);
                if (!blank) {
                    n->text = decode(data);
                    n->has_text = true;
                }
            }
            i = e == std::string::npos ? s.size() : e;
        }
    }
    // the document: its top-level elements
    bool document(std::vector<std::unique_ptr<XNode>>& top) {
        for (;;) {
            skip_ws();
            if (i >= s.size()) return true;
            if (skip_misc()) continue;
            if (s[i] != '<') {
                err = "text outside an XML element";
                return false;
            }
            auto n = element(0);
            if (!n) return false;
            top.push_back(std::move(n));
        }
    }
};

std::string trim(const std::string& v) {
    size_t b = 0, e = v.size();
    while (b < e && std::isspace((unsigned char)v[b])) b++;
    while (e > b && std::isspace((unsigned char)v[e - 1])) e--;
    return v.substr(b, e - b);
}

bool file_exists(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0;
}

// ---------------------------------------------------------------------------
// the nvMatrix / nvVector arithmetic the reference applies to meshes
// ---------------------------------------------------------------------------
struct V3 {
    float x = 0.f, y = 0.f, z = 0.f;
};
struct M4 {
    float m[4][4];  // m[row][col]
    static M4 identity() {
        M4 r;
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) r.m[a][b] = a == b ? 1.f : 0.f;
        return r;
    }
};

// matrix4 * vec4(v, 1), x y z of the result (nvMatrix.h:424-433):
// (((x m0 + y m1) + z m2) + 1 m3) in FP32; host code is built with
// -ffp-contract=off, so nothing is fused
V3 mul_point(const M4& M, const V3& v) {
    float r[3];
    for (int i = 0; i < 3; i++) r[i] = v.x * M.m[i][0] + v.y * M.m[i][1] + v.z * M.m[i][2] + 1.f * M.m[i][3];
    return V3{r[0], r[1], r[2]};
}

// "(x, y, z)" (readVec, config.cpp:620-624): components that do not parse stay 0
V3 read_vec(const char* t) {
    V3 v;
    float f[3] = {0, 0, 0};
    const int n = sscanf(t, " (%f , %f , %f )", &f[0], &f[1], &f[2]);
    if (n >= 1) v.x = f[0];
    if (n >= 2) v.y = f[1];
    if (n >= 3) v.z = f[2];
    return v;
}

// "[a, b, c, d][...]..." row by row (readMatrix, config.cpp:610-619:
// set_value fills columns, transpose turns the text's brackets into rows)
M4 read_matrix(const char* t) {
    float v[16] = {0};
    sscanf(t, " [%f , %f , %f , %f ] [%f , %f , %f , %f ] [%f , %f , %f , %f ] [%f , %f , %f , %f ]", v, v + 1, v + 2,
           v + 3, v + 4, v + 5, v + 6, v + 7, v + 8, v + 9, v + 10, v + 11, v + 12, v + 13, v + 14, v + 15);
    M4 M;
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) M.m[r][c] = v[4 * r + c];
    return M;
}

struct Mesh {
    std::vector<V3> v;
    std::vector<uint32_t> f;  // 3 per face, local vertex indices
    std::string name;
};

// Mesh::getBoundingBox (mesh.cpp:128-142) with the MIN/MAX macros
void bbox(const std::vector<V3>& v, V3& lo, V3& hi) {
    if (v.empty()) return;
    lo = hi = v[0];
    for (size_t k = 1; k < v.size(); k++) {
        const V3& p = v[k];
        lo.x = p.x < lo.x ? p.x : lo.x;
        hi.x = p.x > hi.x ? p.x : hi.x;
        lo.y = p.y < lo.y ? p.y : lo.y;
        hi.y = p.y > hi.y ? p.y : hi.y;
        lo.z = p.z < lo.z ? p.z : lo.z;
        hi.z = p.z > hi.z ? p.z : hi.z;
    }
}

// Mesh::unitize (mesh.cpp:144-158): the vertices in place; returns 2 / maxLen,
// the only part of its matrix that reaches x, y, z
float unitize(std::vector<V3>& v) {
    V3 lo, hi;
    bbox(v, lo, hi);
    V3 c;  // (minCoord + maxCoord) / 2
    c.x = (lo.x + hi.x) / 2.f;
    c.y = (lo.y + hi.y) / 2.f;
    c.z = (lo.z + hi.z) / 2.f;
    const float dx = hi.x - lo.x, dy = hi.y - lo.y, dz = hi.z - lo.z;
    float maxLen = dx < dy ? dy : dx;  // std::max
    maxLen = maxLen < dz ? dz : maxLen;
    const float half = maxLen / 2.f;
    for (auto& p : v) {
        p.x -= c.x;
        p.y -= c.y;
        p.z -= c.z;
        if (half != 0.f) {  // vec3 /= scalar leaves the vector for 0 (nvVector.h:376-380)
            p.x /= half;
            p.y /= half;
            p.z /= half;
        }
    }
    return 2.f / maxLen;
}

struct Loader {
    std::string err;
    std::string root;  // directory of the config file
    std::map<std::string, std::vector<std::unique_ptr<XNode>>> docs;

    // a path as given when it exists or is absolute, else under the config's directory (_access test, config.cpp:630)
    std::string resolve(const std::string& p) const {
        return file_exists(p) || (!p.empty() && p[0] == '/') ? p : root + "/" + p;
    }
    const std::vector<std::unique_ptr<XNode>>* doc(const std::string& path) {
        const std::string full = resolve(path);
        auto it = docs.find(full);
        if (it != docs.end()) return &it->second;
        std::ifstream in(full, std::ios::binary);
        if (!in) {
            err = "cannot open " + full;
            return nullptr;
        }
        std::stringstream ss;
        ss << in.rdbuf();
        const std::string text = ss.str();
        XmlParser p(text);
        std::vector<std::unique_ptr<XNode>> top;
        if (!p.document(top)) {
            err = full + ": " + p.err;
            return nullptr;
        }
        return &(docs[full] = std::move(top));
    }
    // Config::findNode (config.cpp:625-660): the first node with the tag that
    // has no Name attribute, any node when the name is empty, else the first
    // whose Name matches
    static const XNode* pick(const std::vector<const XNode*>& nodes, const std::string& name) {
        for (const XNode* n : nodes) {
            const std::string* a = n->attr("Name");
            if (!a || name.empty()) return n;
            if (*a == name) return n;
        }
        return nullptr;
    }
    const XNode* find_in_file(const std::string& path, const char* tag, const std::string& name) {
        if (path.empty()) return nullptr;
        const auto* top = doc(path);
        if (!top) return nullptr;
        std::vector<const XNode*> cand;
        for (auto& n : *top)
            if (n->tag == tag) cand.push_back(n.get());
        return pick(cand, name);
    }
    static const XNode* find_in_node(const XNode* root, const char* tag, const std::string& name) {
        std::vector<const XNode*> cand;
        for (auto& n : root->kids)
            if (n->tag == tag) cand.push_back(n.get());
        return pick(cand, name);
    }

    // Mesh::loadShape (mesh.cpp:5-127); shapes != nullptr: the "g" groups
    bool load_shape(const std::string& file, Mesh& whole, std::vector<Mesh>* shapes) {
        if (file.size() < 4) {
            err = "mesh file name too short: " + file;
            return false;
        }
        const std::string suffix = file.substr(file.size() - 4);
        if (suffix == ".shp") {
            FILE* fp = fopen(file.c_str(), "rb");
            if (!fp) {
                err = "cannot open " + file;
                return false;
            }
            int32_t n = 0, m = 0;
            bool ok = fread(&n, 4, 1, fp) == 1 && n >= 0 && n <= (1 << 28);
            std::vector<float> vdata(ok ? (size_t)n : 0);
            ok = ok && fread(vdata.data(), 4, vdata.size(), fp) == vdata.size();
            ok = ok && fread(&m, 4, 1, fp) == 1 && m >= 0 && m <= (1 << 28);
            std::vector<uint32_t> fdata(ok ? (size_t)m : 0);
            ok = ok && fread(fdata.data(), 4, fdata.size(), fp) == fdata.size();
            fclose(fp);
            if (!ok) {
                err = "truncated .shp file " + file;
                return false;
            }
            whole.v.assign((size_t)n, V3{});
            for (size_t k = 0; k < vdata.size(); k++) {
                V3& dst = whole.v[k / 3];
                (k % 3 == 0 ? dst.x : (k % 3 == 1 ? dst.y : dst.z)) = vdata[k];
            }
            whole.f.assign(3 * (size_t)m, 0u);
            for (size_t k = 0; k < fdata.size(); k++) whole.f[k] = fdata[k];
        } else if (suffix == ".obj") {
            FILE* fp = fopen(file.c_str(), "r");
            if (!fp) {
                err = "cannot open " + file;
                return false;
            }
            char line[4096];
            Mesh* shape = nullptr;
            uint32_t current_fi = 0;
            bool ok = true;
            while (ok && fgets(line, sizeof line, fp)) {
                if (line[0] == '#') continue;
                char attrib[1024], p0[1024], p1[1024], p2[1024];
                const int num = sscanf(line, "%1023s %1023s %1023s %1023s", attrib, p0, p1, p2);
                if (num >= 1 && !strcmp(attrib, "g") && shapes) {
                    shapes->emplace_back();
                    shape = &shapes->back();
                    shape->name = num >= 2 ? p0 : "";
                    current_fi = (uint32_t)whole.v.size();
                }
                if (num != 4) continue;
                if (!strcmp(attrib, "v")) {
                    V3 p;
                    p.x = strtof(p0, nullptr);
                    p.y = strtof(p1, nullptr);
                    p.z = strtof(p2, nullptr);
                    whole.v.push_back(p);
                    if (shape) shape->v.push_back(p);
                } else if (!strcmp(attrib, "f")) {
                    uint32_t t[3];
                    const char* ps[3] = {p0, p1, p2};
                    for (int k = 0; k < 3 && ok; k++) {
                        char* end = nullptr;
                        const long x = strtol(ps[k], &end, 10);
                        if (end == ps[k] || x < 1) {
                            err = "unsupported face index in " + file + ": " + ps[k];
                            ok = false;
                        }
                        t[k] = (uint32_t)(x - 1);
                    }
                    if (!ok) break;
                    for (int k = 0; k < 3; k++) whole.f.push_back(t[k]);
                    if (shape)
                        for (int k = 0; k < 3; k++) shape->f.push_back(t[k] - current_fi);
                }
            }
            fclose(fp);
            if (!ok) return false;
        } else {
            err = "unknown mesh format (.obj or .shp): " + file;
            return false;
        }
        auto check = [&](const Mesh& m) {
            for (uint32_t x : m.f)
                if (x >= m.v.size()) {
                    err = "face index out of range in " + file + (m.name.empty() ? "" : " (group " + m.name + ")");
                    return false;
                }
            return true;
        };
        if (!check(whole)) return false;
        if (shapes)
            for (auto& s : *shapes)
                if (!check(s)) return false;
        return true;
    }
};

}  // namespace

struct wr_scene_file {
    std::vector<wr_object_desc> objects;
    std::vector<float> vertices;
    std::vector<uint32_t> triangles;
    std::vector<wr_grid_desc> grids;
    std::vector<std::vector<float>> grid_data;
    wr_camera_desc camera{};
    char renderer[32] = {0};
    uint32_t spp = 0, max_path_len = 20;
    float radius = 0.f;
    uint32_t mode = 0xffffffffu;
};

namespace {

void set3(float* d, const V3& v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

bool child_float(const XNode* n, const char* tag, float* out) {
    const XNode* k = n->first(tag);
    if (!k) return false;
    *out = (float)atof(k->value());
    return true;
}

// a <Material> onto an object description (generateSceneObject, config.cpp:21-430)
bool material(Loader& L, const XNode* mat, wr_object_desc& d, std::string* grid_file) {
    const XNode* tn = mat->first("type");
    const std::string type = tn ? trim(tn->value()) : "";
    d.ior = 1.5f;  // RefractiveObject / HeterogeneousVolume defaults
    set3(d.decay, V3{1, 1, 1});
    d.density_scale = 100.f;
    d.step_size = 0.002f;
    d.grid_index = 0xffffffffu;
    if (type == "Diffuse" || type == "Glossy" || type == "Emissive") {
        const XNode* c = mat->first("color");
        if (!c) {
            L.err = type + " material without <color>";
            return false;
        }
        if (type == "Emissive") {
            d.type = WR_MAT_EMISSIVE;
            set3(d.emission, read_vec(c->value()));
        } else {
            d.type = type == "Diffuse" ? WR_MAT_DIFFUSE : WR_MAT_GLOSSY;
            set3(d.albedo, read_vec(c->value()));
        }
        if (type == "Glossy" && !child_float(mat, "power", &d.power)) {
            L.err = "Glossy material without <power>";
            return false;
        }
        return true;
    }
    if (type == "Reflective") {
        d.type = WR_MAT_REFLECTIVE;
        const XNode* c = mat->first("color");
        set3(d.albedo, c ? read_vec(c->value()) : V3{1, 1, 1});  // reflectiveObj.h:10
        return true;
    }
    if (type == "Refractive") {
        d.type = WR_MAT_REFRACTIVE;
        child_float(mat, "IOR", &d.ior);
        if (const XNode* c = mat->first("decayColor")) set3(d.decay, read_vec(c->value()));
        return true;
    }
    if (type == "AnisotropicGlossy") {
        d.type = WR_MAT_ANISO;
        const XNode *rs = mat->first("Rs"), *rd = mat->first("Rd");
        if (!rs || !rd || !child_float(mat, "Nu", &d.nu) || !child_float(mat, "Nv", &d.nv)) {
            L.err = "AnisotropicGlossy material needs <Rs> <Rd> <Nu> <Nv>";
            return false;
        }
        set3(d.rs, read_vec(rs->value()));
        set3(d.rd, read_vec(rd->value()));
        return true;
    }
    if (type == "Volume" || type == "GridVolume") {
        d.type = type == "Volume" ? WR_MAT_HOMOGENEOUS : WR_MAT_HETEROGENEOUS;
        if (!child_float(mat, "g", &d.g)) {
            L.err = type + " material without <g>";
            return false;
        }
        // a homogeneous volume without <IOR> has an uninitialised IOR in the reference; 1 here
        if (type == "Volume") d.ior = 1.f;
        child_float(mat, "IOR", &d.ior);
        child_float(mat, "stepsize", &d.step_size);
        const XNode *ss = mat->first("sigma_s"), *sa = mat->first("sigma_a");
        if (ss && sa) {
            set3(d.sigma_s, read_vec(ss->value()));
            set3(d.sigma_a, read_vec(sa->value()));
        }
        if (type == "GridVolume") {
            child_float(mat, "density_scale", &d.density_scale);
            float sub = 0.f;
            if ((child_float(mat, "subsurface", &sub) && sub != 0.f) || mat->first("volume_data_s")) {
                L.err = "subsurface grid volumes are not supported";
                return false;
            }
            const XNode* df = mat->first("density_file");
            if (!df) {
                L.err = "GridVolume material without <density_file>";
                return false;
            }
            *grid_file = trim(df->value());
        }
        return true;
    }
    L.err = type.empty() ? std::string("material without <type>") : "material type not supported: " + type;
    return false;
}

// HeterogeneousVolume::loadDensityMap (HeterogeneousVolume.cpp:12-39): text
// "nx ny nz" then nx*ny*nz values, z-major; the grid spans the mesh's box
bool load_grid(Loader& L, const std::string& file, wr_scene_file& out, const std::vector<V3>& local, const M4& T,
               uint32_t* index) {
    std::ifstream in(L.resolve(file));
    if (!in) {
        L.err = "cannot open density file " + file;
        return false;
    }
    long long nx = 0, ny = 0, nz = 0;
    if (!(in >> nx >> ny >> nz) || nx < 1 || ny < 1 || nz < 1 || nx * ny * nz > (1ll << 31)) {
        L.err = "bad density file header " + file;
        return false;
    }
    std::vector<float> data((size_t)(nx * ny * nz));
    for (auto& x : data)
        if (!(in >> x)) {
            L.err = "truncated density file " + file;
            return false;
        }
    // the reference looks the grid up in the object's local box; the device
    // grid is axis-aligned in world space, so the transform must not rotate
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            if (r != c && T.m[r][c] != 0.f) {
                L.err = "a GridVolume's transform must not rotate (the grid is axis-aligned)";
                return false;
            }
    V3 lo, hi;
    bbox(local, lo, hi);
    const V3 a = mul_point(T, lo), b = mul_point(T, hi);
    wr_grid_desc g{};
    g.nx = (uint32_t)nx;
    g.ny = (uint32_t)ny;
    g.nz = (uint32_t)nz;
    g.p0[0] = std::fmin(a.x, b.x);
    g.p0[1] = std::fmin(a.y, b.y);
    g.p0[2] = std::fmin(a.z, b.z);
    g.p1[0] = std::fmax(a.x, b.x);
    g.p1[1] = std::fmax(a.y, b.y);
    g.p1[2] = std::fmax(a.z, b.z);
    out.grid_data.push_back(std::move(data));
    out.grids.push_back(g);
    *index = (uint32_t)out.grids.size() - 1;
    return true;
}

bool add_object(Loader& L, wr_scene_file& out, const XNode* obj_node, const XNode* mat, const Mesh& mesh,
                const M4& T) {
    wr_object_desc d{};
    std::string grid_file;
    if (!material(L, mat, d, &grid_file)) return false;
    if (obj_node->first("motion")) {
        L.err = "<motion> is not supported (the reference renders one random instant per object)";
        return false;
    }
    d.vert_begin = (uint32_t)(out.vertices.size() / 3);
    d.vert_count = (uint32_t)mesh.v.size();
    d.tri_begin = (uint32_t)(out.triangles.size() / 3);
    d.tri_count = (uint32_t)(mesh.f.size() / 3);
    for (const V3& p : mesh.v) {
        const V3 w = mul_point(T, p);
        out.vertices.push_back(w.x);
        out.vertices.push_back(w.y);
        out.vertices.push_back(w.z);
    }
    out.triangles.insert(out.triangles.end(), mesh.f.begin(), mesh.f.end());
    if (d.type == WR_MAT_HETEROGENEOUS && !load_grid(L, grid_file, out, mesh.v, T, &d.grid_index)) return false;
    out.objects.push_back(d);
    return true;
}

// Config::getPathAndName (config.cpp:661-666)
std::pair<std::string, std::string> path_and_name(const XNode* n, const std::string& current) {
    const XNode* p = n->first("path");
    const XNode* m = n->first("name");
    return {p ? trim(p->value()) : current, m ? trim(m->value()) : std::string()};
}

int load(const char* config_path, wr_scene_file* out, std::string& err) {
    Loader L;
    const std::string cfg = config_path;
    const size_t pos = cfg.find_last_of("/\\");
    L.root = pos == std::string::npos ? std::string(".") : cfg.substr(0, pos);
    const XNode* config = L.find_in_file(cfg, "Config", "");
    if (!config) {
        err = L.err.empty() ? "no <Config> in " + cfg : L.err;
        return WR_ERR_INVALID_ARGUMENT;
    }
    const XNode* scene_cfg = config->first("Scene");
    if (!scene_cfg) {
        err = "<Config> without <Scene>";
        return WR_ERR_INVALID_ARGUMENT;
    }
    auto pn = path_and_name(scene_cfg, "");
    const XNode* scene = L.find_in_file(pn.first, "Scene", pn.second);
    std::string first_err;
    if (!scene) {  // the reference then looks in the config file itself
        first_err = L.err;
        L.err.clear();
        scene = L.find_in_file(cfg, "Scene", pn.second);
    }
    if (!scene) {
        err = !first_err.empty() ? first_err : (L.err.empty() ? "scene " + pn.second + " not found" : L.err);
        return WR_ERR_INVALID_ARGUMENT;
    }
    const std::string current = pn.first.empty() ? cfg : pn.first;
    auto material_of = [&](const XNode* obj) -> const XNode* {
        const XNode* m = obj->first("Material");
        if (!m) {
            L.err = "<Object> without <Material>";
            return nullptr;
        }
        auto mp = path_and_name(m, current);
        const XNode* mat = L.find_in_file(mp.first, "Material", mp.second);
        if (!mat && L.err.empty()) L.err = "material " + mp.second + " not found";
        return mat;
    };
    // group objects first, as Config::load reads them (config.cpp:456-490)
    for (auto& gk : scene->kids) {
        if (gk->tag != "GroupObject") continue;
        const XNode* fp = gk->first("filePath");
        if (!fp) {
            err = "<GroupObject> without <filePath>";
            return WR_ERR_INVALID_ARGUMENT;
        }
        const std::string path = L.resolve(trim(fp->value()));
        M4 gT = M4::identity();
        if (const XNode* t = gk->first("transform")) gT = read_matrix(t->value());
        Mesh whole;
        std::vector<Mesh> shapes;
        if (!L.load_shape(path, whole, &shapes)) {
            err = L.err;
            return WR_ERR_INVALID_ARGUMENT;
        }
        // unitize the whole mesh; its matrix only scales the shapes (see the header)
        const float s = unitize(whole.v);
        M4 U = M4::identity();
        U.m[0][0] = U.m[1][1] = U.m[2][2] = s;
        for (auto& sh : shapes)
            for (auto& p : sh.v) p = mul_point(U, p);
        for (auto& ok : gk->kids) {
            if (ok->tag != "Object") continue;
            const std::string* nm = ok->attr("Name");
            const Mesh* shape = nullptr;
            for (auto& sh : shapes)
                if (nm && sh.name == *nm) shape = &sh;  // name_shape map: the last group of a name wins
            const XNode* mat = material_of(ok.get());
            if (!mat) {
                err = L.err;
                return WR_ERR_INVALID_ARGUMENT;
            }
            bool added;
            if (shape) {
                added = add_object(L, *out, ok.get(), mat, *shape, gT);
            } else {
                Mesh all;
                M4 T = M4::identity();
                if (const XNode* t = ok->first("transform")) T = read_matrix(t->value());
                added = L.load_shape(path, all, nullptr);
                if (added) {
                    unitize(all.v);
                    added = add_object(L, *out, ok.get(), mat, all, T);
                }
            }
            if (!added) {
                err = L.err;
                return WR_ERR_INVALID_ARGUMENT;
            }
        }
    }
    for (auto& ok : scene->kids) {
        if (ok->tag != "Object") continue;
        const XNode* fp = ok->first("filePath");
        if (!fp) {
            err = "<Object> without <filePath>";
            return WR_ERR_INVALID_ARGUMENT;
        }
        const std::string path = L.resolve(trim(fp->value()));
        const XNode* mat = material_of(ok.get());
        if (!mat) {
            err = L.err;
            return WR_ERR_INVALID_ARGUMENT;
        }
        M4 T = M4::identity();
        if (const XNode* t = ok->first("transform")) T = read_matrix(t->value());
        Mesh mesh;
        if (!L.load_shape(path, mesh, nullptr)) {
            err = L.err;
            return WR_ERR_INVALID_ARGUMENT;
        }
        unitize(mesh.v);
        if (!add_object(L, *out, ok.get(), mat, mesh, T)) {
            err = L.err;
            return WR_ERR_INVALID_ARGUMENT;
        }
    }
    // camera (config.cpp:510-524)
    const XNode* camname = scene_cfg->first("camera");
    const XNode* cam = Loader::find_in_node(scene, "Camera", camname ? trim(camname->value()) : std::string());
    if (!cam) {
        err = "camera not found";
        return WR_ERR_INVALID_ARGUMENT;
    }
    for (const char* k : {"position", "focus", "up", "width", "height", "sightDist"})
        if (!cam->first(k)) {
            err = std::string("<Camera> without <") + k + ">";
            return WR_ERR_INVALID_ARGUMENT;
        }
    wr_camera_desc& c = out->camera;
    set3(c.position, read_vec(cam->first("position")->value()));
    set3(c.focus, read_vec(cam->first("focus")->value()));
    set3(c.up, read_vec(cam->first("up")->value()));
    const float w = (float)atof(cam->first("width")->value()), h = (float)atof(cam->first("height")->value());
    if (!(w >= 1.f && h >= 1.f && w < 65536.f && h < 65536.f)) {
        err = "camera width and height must be between 1 and 65535";
        return WR_ERR_INVALID_ARGUMENT;
    }
    c.width = (uint32_t)w;
    c.height = (uint32_t)h;
    c.image_plane_dist = (float)atof(cam->first("sightDist")->value());
    c.lens_radius = 0.f;
    c.focal_dist = 3.402823466e+38f;
    if (cam->first("lensRadius") && cam->first("focalDist")) {
        c.lens_radius = (float)atof(cam->first("lensRadius")->value());
        c.focal_dist = (float)atof(cam->first("focalDist")->value());
    }
    // renderer (config.cpp:535-573): the name, spp from <iter>, path length 20
    if (const XNode* r = config->first("renderer"))
        snprintf(out->renderer, sizeof out->renderer, "%s", trim(r->value()).c_str());
    out->spp = 0;
    if (const XNode* it = config->first("iter")) {
        const double v = atof(it->value());
        out->spp = v > 0 ? (uint32_t)std::fmin(v, 4294967295.0) : 0u;
    }
    out->max_path_len = 20;
    // <radius> of VCMTracer / PhotonMap (config.cpp:560, 571: setRadius(atof(...)))
    out->radius = 0.f;
    if (const XNode* rr = config->first("radius")) out->radius = (float)atof(rr->value());
    const std::string name = out->renderer;
    out->mode = (name == "PathTracer" || name == "PT")             ? WR_MODE_WAVEFRONT
                : (name == "BidirPathTracer" || name == "BPT") ? WR_MODE_BIDIRECTIONAL
                : (name == "VCMTracer" || name == "VCM")       ? WR_MODE_VCM
                : (name == "PhotonMap" || name == "PM")        ? WR_MODE_PHOTON_MAP
                                                               : 0xffffffffu;
    for (size_t k = 0; k < out->grids.size(); k++) out->grids[k].density = out->grid_data[k].data();
    return WR_OK;
}

}  // namespace

extern "C" {

int wr_scene_file_load(const char* config_path, wr_scene_file** out, char* err, size_t err_len) {
    if (err && err_len) err[0] = 0;
    if (!config_path || !out) return WR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::string msg;
    try {
        auto f = std::make_unique<wr_scene_file>();
        const int rc = load(config_path, f.get(), msg);
        if (rc != WR_OK) {
            if (err && err_len) snprintf(err, err_len, "%s", msg.c_str());
            return rc;
        }
        *out = f.release();
        return WR_OK;
    } catch (const std::bad_alloc&) {
        if (err && err_len) snprintf(err, err_len, "out of host memory");
        return WR_ERR_OUT_OF_MEMORY;
    } catch (...) {
        if (err && err_len) snprintf(err, err_len, "scene file loader failed");
        return WR_ERR_INTERNAL;
    }
}

int wr_scene_file_get(const wr_scene_file* f, wr_scene_desc* desc, wr_scene_file_settings* settings) {
    if (!f) return WR_ERR_INVALID_ARGUMENT;
    if (desc) {
        desc->num_objects = (uint32_t)f->objects.size();
        desc->num_vertices = (uint32_t)(f->vertices.size() / 3);
        desc->num_triangles = (uint32_t)(f->triangles.size() / 3);
        desc->num_grids = (uint32_t)f->grids.size();
        desc->objects = f->objects.data();
        desc->vertices = f->vertices.data();
        desc->triangles = f->triangles.data();
        desc->grids = f->grids.data();
        desc->camera = f->camera;
    }
    if (settings) {
        memcpy(settings->renderer, f->renderer, sizeof settings->renderer);
        settings->spp = f->spp;
        settings->max_path_len = f->max_path_len;
        settings->radius = f->radius;
        settings->mode = f->mode;
    }
    return WR_OK;
}

int wr_scene_file_free(wr_scene_file* f) {
    delete f;
    return WR_OK;
}

}  // extern "C"
