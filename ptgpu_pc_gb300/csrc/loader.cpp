// loader.cpp -- scene files, camera and seeds (host side).
//
// read_scene keeps the reference loader's behaviour (displayfunc.cpp:144-730):
//   .txt  ReadTxt: gamma/sky line (optional), camera eye/target, material
//         descriptors, then `objects N` lines of sphere / triangle / model
//         (OBJ, scaled then translated); area and light count are computed
//         as the reference does; walllight becomes false.
//   .scn  ReadScene: camera, `size N`, N sphere lines; area and light count
//         are left unset (0) as in the reference, and walllight stays true so
//         the caller appends AddWallLight's nine spheres.
//   .ply  not supported (the reference delegates to a third-party reader).
// The format strings below are the scene-file grammar and therefore match the
// reference's; the OBJ reader is this library's own (v and f records, the
// reference reader's line rule; faces with more than three vertices are
// fanned into triangles).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <algorithm>
#include <thread>
#include <vector>

#include "host.h"

namespace ptgpu {

namespace {

constexpr float kPiF = 3.14159265358979323846f;

enum { MAT_LAMBERTIAN = 0, MAT_CONDUCTOR, MAT_DIELECTRIC, MAT_MATTE, MAT_PLASTIC, MAT_METAL };

int refl_from_material(int mat) {
    if (mat == MAT_LAMBERTIAN) return PTGPU_DIFF;
    if (mat == MAT_CONDUCTOR) return PTGPU_SPEC;
    if (mat == MAT_DIELECTRIC) return PTGPU_REFR;
    return PTGPU_DIFF;   // MATTE / PLASTIC / METAL are parsed but shaded as DIFF
}

bool viszero(const ptgpu_vec &v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }

// |cross(p2-p1, p3-p1)| * 0.5f (displayfunc.cpp:315-318)
float triangle_area(const ptgpu_vec &p1, const ptgpu_vec &p2, const ptgpu_vec &p3) {
    ptgpu_vec e1 = {p2.x - p1.x, p2.y - p1.y, p2.z - p1.z};
    ptgpu_vec e2 = {p3.x - p1.x, p3.y - p1.y, p3.z - p1.z};
    ptgpu_vec n = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    return sqrtf(n.x * n.x + n.y * n.y + n.z * n.z) * 0.5f;
}

// parses one face vertex token "i", "i/j", "i//k" or "i/j/k" -> 0-based index
bool face_index(const char *tok, int32_t nverts, int32_t *out) {
    char *end = nullptr;
    long i = std::strtol(tok, &end, 10);
    if (end == tok) return false;
    if (i < 0) i = nverts + i;     // relative index
    else i = i - 1;
    if (i < 0 || i >= nverts) return false;
    *out = (int32_t)i;
    return true;
}

// Kind of one OBJ line (a NUL-terminated copy, so that sscanf and strtok_r
// see exactly the line): 0 other, 1 vertex, 2 face.
int obj_line_kind(const char *p) {
    while (*p == ' ' || *p == '\t') ++p;
    if (p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) return 1;
    if (p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) return 2;
    return 0;
}

// The file is split into lines the way the reference's OBJ reader does: the
// buffer's last byte is taken for a terminator, so only lines ended by '\n',
// '\0' or a lone '\r' before the final byte count (a file whose last line is
// followed by a single newline loses that line, as in the reference scenes).
inline bool obj_term(const std::string &buf, size_t i, size_t end_idx) {
    const char ch = buf[i];
    return ch == '\0' || ch == '\n' || (ch == '\r' && i + 1 < end_idx && buf[i + 1] != '\n');
}

// A run of whole lines [begin, end) of the file (end is just past a
// terminator, or the file's end index for the last run).
struct ObjRun {
    size_t begin = 0, end = 0;
    int64_t nv = 0, ntri = 0;        // vertex lines; triangles after fanning
    int64_t v0 = 0, t0 = 0;          // vertices and triangles before the run
    bool ok = true;
    int bad_kind = 0;                // the first malformed line: 1 vertex, 2 face
};

// Counts vertex lines and fanned triangles of a run.
void obj_count(const std::string &buf, size_t end_idx, ObjRun &r) {
    size_t prev = r.begin;
    for (size_t i = r.begin; i < r.end && i < end_idx; ++i) {
        if (!obj_term(buf, i, end_idx)) continue;
        const char *p = buf.data() + prev;
        const char *q = buf.data() + i;
        prev = i + 1;
        while (p < q && (*p == ' ' || *p == '\t')) ++p;
        if (q - p < 2 || (p[1] != ' ' && p[1] != '\t')) continue;
        if (p[0] == 'v') {
            ++r.nv;
        } else if (p[0] == 'f') {
            int64_t tok = 0;
            bool in = false;
            for (const char *c = p + 2; c < q; ++c) {
                const bool sep = *c == ' ' || *c == '\t' || *c == '\r' || *c == '\n' || *c == '\0';
                if (!sep && !in) ++tok;
                in = !sep;
                if (*c == '\0') break;          // strtok_r stops at the copy's end
            }
            if (tok > 2) r.ntri += tok - 2;
        }
    }
}

// Parses a run into obj.v / obj.tri at the run's vertex and triangle bases.
void obj_parse(const std::string &buf, size_t end_idx, ObjRun &r, Obj &obj) {
    std::string line;
    std::vector<int32_t> face;
    int64_t nv = r.v0, nt = r.t0;
    size_t prev = r.begin;
    for (size_t i = r.begin; i < r.end && i < end_idx; ++i) {
        if (!obj_term(buf, i, end_idx)) continue;
        line.assign(buf, prev, i - prev);
        prev = i + 1;
        const int kind = obj_line_kind(line.c_str());
        if (kind == 0) continue;
        const char *p = line.c_str();
        while (*p == ' ' || *p == '\t') ++p;
        if (kind == 1) {
            float x, y, z;
            if (std::sscanf(p + 2, "%f %f %f", &x, &y, &z) != 3) { r.ok = false; r.bad_kind = 1; return; }
            obj.v[3 * nv] = x; obj.v[3 * nv + 1] = y; obj.v[3 * nv + 2] = z;
            ++nv;
        } else {
            face.clear();
            std::string rest(p + 2);
            char *save = nullptr;
            for (char *tok = strtok_r(&rest[0], " \t\r\n", &save); tok; tok = strtok_r(nullptr, " \t\r\n", &save)) {
                int32_t idx;
                if (!face_index(tok, (int32_t)nv, &idx)) { r.ok = false; r.bad_kind = 2; return; }
                face.push_back(idx);
            }
            for (size_t k = 2; k < face.size(); ++k) {
                obj.tri[3 * nt] = face[0]; obj.tri[3 * nt + 1] = face[k - 1]; obj.tri[3 * nt + 2] = face[k];
                ++nt;
            }
        }
    }
}

}  // namespace

// The whole file is read once; runs of lines are then counted and parsed on
// up to `threads` host threads (one run per thread, cut at line ends), each
// run writing its vertices and triangles at bases known from the counts, so
// the result is the sequential reader's: same vertices, same triangles in
// file order, same errors (a face may only use vertices defined above it).
bool read_obj(const char *path, Obj &obj, std::string &err, int threads) {
    FILE *f = std::fopen(path, "rb");
    if (!f) { err = std::string("cannot open model ") + path; return false; }
    std::string buf;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long sz = std::ftell(f);
        if (sz > 0) buf.reserve((size_t)sz);
        std::fseek(f, 0, SEEK_SET);
    }
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.append(chunk, got);
    std::fclose(f);
    if (buf.empty()) { err = "empty model " + std::string(path); return false; }
    const size_t end_idx = buf.size() - 1;
    if (threads <= 0) {
        const unsigned hw = std::thread::hardware_concurrency();
        threads = (int)std::min<size_t>(std::max(1u, std::min(hw, 16u)), std::max<size_t>(1, buf.size() >> 20));
    }
    // runs cut just past a terminator
    std::vector<ObjRun> runs;
    size_t start = 0;
    for (int t = 0; t < threads && start < end_idx; ++t) {
        size_t stop = end_idx;
        if (t + 1 < threads) {
            size_t i = std::max(start, (size_t)((double)end_idx * (t + 1) / threads));
            while (i < end_idx && !obj_term(buf, i, end_idx)) ++i;
            stop = i < end_idx ? i + 1 : end_idx;
        }
        ObjRun r;
        r.begin = start;
        r.end = stop;
        runs.push_back(r);
        start = stop;
    }
    // runs on their own threads; a run whose thread cannot be started is
    // done on this one (no exception leaves the reader)
    auto for_runs = [&](auto fn) {
        std::vector<std::thread> th;
        std::vector<char> started(runs.size(), 0);
        for (size_t k = 1; k < runs.size(); ++k) {
            try {
                th.emplace_back([&, k] { fn(runs[k]); });
                started[k] = 1;
            } catch (...) {
            }
        }
        if (!runs.empty()) fn(runs[0]);
        for (auto &x : th) x.join();
        for (size_t k = 1; k < runs.size(); ++k)
            if (!started[k]) fn(runs[k]);
    };
    for_runs([&](ObjRun &r) { obj_count(buf, end_idx, r); });
    int64_t nv = 0, nt = 0;
    for (ObjRun &r : runs) { r.v0 = nv; r.t0 = nt; nv += r.nv; nt += r.ntri; }
    obj.v.assign((size_t)(3 * nv), 0.f);
    obj.tri.assign((size_t)(3 * nt), 0);
    for_runs([&](ObjRun &r) { obj_parse(buf, end_idx, r, obj); });
    for (const ObjRun &r : runs) {       // the first malformed line in file order
        if (r.ok) continue;
        err = (r.bad_kind == 1 ? "malformed vertex in " : "malformed face in ") + std::string(path);
        return false;
    }
    return true;
}

namespace {

ptgpu_shape sphere_shape(float rad, ptgpu_vec c, ptgpu_vec e, ptgpu_vec col, int refl) {
    ptgpu_shape s;
    std::memset(&s, 0, sizeof(s));
    s.type = PTGPU_SPHERE;
    s.g.s.rad = rad;
    s.g.s.p = c;
    s.e = e;
    s.c = col;
    s.refl = refl;
    return s;
}

std::string dir_of(const char *path) {
    const char *slash = std::strrchr(path, '/');
    return slash ? std::string(path, slash - path + 1) : std::string();
}

// Receives the objects of a .txt scene in file order.
struct TxtSink {
    virtual ~TxtSink() = default;
    virtual void shape(const ptgpu_shape &s) = 0;
    virtual void model(Obj &&obj, ptgpu_vec pos, ptgpu_vec scale, ptgpu_vec e, ptgpu_vec col, int refl) = 0;
};

// model triangles as shapes (displayfunc.cpp:395-420): scale then translate
ptgpu_shape model_triangle(const Obj &obj, size_t t, ptgpu_vec pos, ptgpu_vec scale, ptgpu_vec e,
                           ptgpu_vec col, int refl) {
    ptgpu_shape s;
    std::memset(&s, 0, sizeof(s));
    s.type = PTGPU_TRIANGLE;
    ptgpu_vec *pv[3] = {&s.g.t.p1, &s.g.t.p2, &s.g.t.p3};
    for (int k = 0; k < 3; ++k) {
        const float *v = &obj.v[3 * (size_t)obj.tri[3 * t + k]];
        pv[k]->x = v[0] * scale.x + pos.x;
        pv[k]->y = v[1] * scale.y + pos.y;
        pv[k]->z = v[2] * scale.z + pos.z;
    }
    s.e = e;
    s.c = col;
    s.refl = refl;
    s.area = triangle_area(s.g.t.p1, s.g.t.p2, s.g.t.p3);
    return s;
}

int parse_txt(const char *path, int width, int height, ptgpu_camera &cam, uint32_t &light_cnt, TxtSink &sink,
              std::string &err) {
    FILE *f = std::fopen(path, "r");
    if (!f) { err = std::string("cannot open scene ") + path; return PTGPU_E_IO; }
    float gamma, sky[6];
    (void)std::fscanf(f, "gamma %f  sky1 %f %f %f  sky2 %f %f %f\n", &gamma, &sky[0], &sky[1],
                      &sky[2], &sky[3], &sky[4], &sky[5]);
    std::memset(&cam, 0, sizeof(cam));
    int c = std::fscanf(f, "camera %f %f %f  %f %f %f\n", &cam.orig.x, &cam.orig.y, &cam.orig.z,
                        &cam.target.x, &cam.target.y, &cam.target.z);
    cam.pitch = 0.f;
    cam.yaw = 0.f;
    cam.width = (float)width;
    cam.height = (float)height;
    if (c != 6) { std::fclose(f); err = "failed to read 6 camera parameters"; return PTGPU_E_IO; }
    unsigned mat_count = 0;
    if (std::fscanf(f, "materials %u\n", &mat_count) < 1) {
        std::fclose(f); err = "failed to read the number of materials"; return PTGPU_E_IO;
    }
    for (unsigned m = 0; m < mat_count; ++m) {   // parsed and discarded (shaded as DIFF)
        char kind[100];
        if (std::fscanf(f, "%99s", kind) != 1) { std::fclose(f); err = "bad material"; return PTGPU_E_IO; }
        float vals[7];
        if (!std::strcmp(kind, "matte")) {
            if (std::fscanf(f, "%f %f %f  %f\n", &vals[0], &vals[1], &vals[2], &vals[3]) != 4) {
                std::fclose(f); err = "bad matte material"; return PTGPU_E_IO;
            }
        } else if (!std::strcmp(kind, "plastic")) {
            if (std::fscanf(f, "%f %f %f  %f %f %f  %f\n", &vals[0], &vals[1], &vals[2], &vals[3],
                            &vals[4], &vals[5], &vals[6]) != 7) {
                std::fclose(f); err = "bad plastic material"; return PTGPU_E_IO;
            }
        }
    }
    unsigned nobj = 0;
    if (std::fscanf(f, "objects %u\n", &nobj) < 1) {
        std::fclose(f); err = "failed to read object count"; return PTGPU_E_IO;
    }
    const std::string base = dir_of(path);
    uint32_t lights = 0;
    for (unsigned li = 0; li < nobj; ++li) {
        char kind[100];
        if (std::fscanf(f, "%99s", kind) != 1) { std::fclose(f); err = "bad object type"; return PTGPU_E_IO; }
        unsigned mat = 0;
        if (!std::strcmp(kind, "sphere")) {
            float r;
            ptgpu_vec cen, e, col;
            int rc = std::fscanf(f, "%f  %f %f %f  %f %f %f  %f %f %f  %u\n", &r, &cen.x, &cen.y,
                                 &cen.z, &e.x, &e.y, &e.z, &col.x, &col.y, &col.z, &mat);
            if (rc != 11 || mat > 5) { std::fclose(f); err = "bad sphere"; return PTGPU_E_IO; }
            ptgpu_shape s = sphere_shape(r, cen, e, col, refl_from_material((int)mat));
            s.area = 4 * kPiF * r * r;
            if (!viszero(e)) ++lights;
            sink.shape(s);
        } else if (!std::strcmp(kind, "triangle")) {
            ptgpu_shape s;
            std::memset(&s, 0, sizeof(s));
            s.type = PTGPU_TRIANGLE;
            int imat = 0;
            int rc = std::fscanf(f, "%f %f %f  %f %f %f  %f %f %f  %f %f %f  %f %f %f  %d\n",
                                 &s.g.t.p1.x, &s.g.t.p1.y, &s.g.t.p1.z, &s.g.t.p2.x, &s.g.t.p2.y,
                                 &s.g.t.p2.z, &s.g.t.p3.x, &s.g.t.p3.y, &s.g.t.p3.z, &s.e.x, &s.e.y,
                                 &s.e.z, &s.c.x, &s.c.y, &s.c.z, &imat);
            if (rc != 16 || imat < 0 || imat > 5) { std::fclose(f); err = "bad triangle"; return PTGPU_E_IO; }
            s.refl = refl_from_material(imat);
            s.area = triangle_area(s.g.t.p1, s.g.t.p2, s.g.t.p3);
            if (!viszero(s.e)) ++lights;
            sink.shape(s);
        } else if (!std::strcmp(kind, "model")) {
            char model[200];
            ptgpu_vec pos, scale, e, col;
            int imat = 0;
            int rc = std::fscanf(f, "%199s  %f %f %f  %f %f %f  %f %f %f  %f %f %f  %d\n", model,
                                 &pos.x, &pos.y, &pos.z, &scale.x, &scale.y, &scale.z, &e.x, &e.y,
                                 &e.z, &col.x, &col.y, &col.z, &imat);
            if (rc != 14 || imat < 0 || imat > 5) { std::fclose(f); err = "bad model"; return PTGPU_E_IO; }
            Obj obj;
            std::string mp = model;
            if (!read_obj(mp.c_str(), obj, err)) {
                // model paths are relative to the working directory in the
                // reference; fall back to the scene file's directory's parent
                std::string alt = base + "../" + mp;
                std::string err2;
                if (!read_obj(alt.c_str(), obj, err2)) { std::fclose(f); return PTGPU_E_IO; }
                err.clear();
            }
            const size_t ntri = obj.tri.size() / 3;
            if (!viszero(e)) lights += (uint32_t)ntri;
            sink.model(std::move(obj), pos, scale, e, col, refl_from_material(imat));
        } else {
            std::fclose(f);
            err = std::string("unknown object type ") + kind;
            return PTGPU_E_IO;
        }
    }
    std::fclose(f);
    light_cnt = lights;
    return PTGPU_OK;
}

struct AosSink : TxtSink {
    std::vector<ptgpu_shape> &out;
    explicit AosSink(std::vector<ptgpu_shape> &o) : out(o) {}
    void shape(const ptgpu_shape &s) override { out.push_back(s); }
    void model(Obj &&obj, ptgpu_vec pos, ptgpu_vec scale, ptgpu_vec e, ptgpu_vec col, int refl) override {
        for (size_t t = 0; t < obj.tri.size() / 3; ++t) out.push_back(model_triangle(obj, t, pos, scale, e, col, refl));
    }
};

struct CompactSink : TxtSink {
    CompactScene &out;
    explicit CompactSink(CompactScene &o) : out(o) {}
    void shape(const ptgpu_shape &s) override {
        if (out.segs.empty() || out.segs.back().model) out.segs.emplace_back();
        out.segs.back().shapes.push_back(s);
    }
    void model(Obj &&obj, ptgpu_vec pos, ptgpu_vec scale, ptgpu_vec e, ptgpu_vec col, int refl) override {
        if (obj.tri.empty()) return;
        out.segs.emplace_back();
        SceneSegment &g = out.segs.back();
        g.model = true;
        g.obj = std::move(obj);
        g.pos = pos; g.scale = scale; g.e = e; g.c = col; g.refl = refl;
    }
};

int read_txt(const char *path, int width, int height, LoadedScene &sc, std::string &err) {
    AosSink sink(sc.shapes);
    int st = parse_txt(path, width, height, sc.camera, sc.light_cnt, sink, err);
    sc.walllight = false;
    return st;
}

int read_scn(const char *path, int width, int height, LoadedScene &sc, std::string &err) {
    FILE *f = std::fopen(path, "r");
    if (!f) { err = std::string("cannot open scene ") + path; return PTGPU_E_IO; }
    ptgpu_camera &cam = sc.camera;
    std::memset(&cam, 0, sizeof(cam));
    int c = std::fscanf(f, "camera %f %f %f %f %f %f\n", &cam.orig.x, &cam.orig.y, &cam.orig.z,
                        &cam.target.x, &cam.target.y, &cam.target.z);
    cam.width = (float)width;
    cam.height = (float)height;
    if (c != 6) { std::fclose(f); err = "failed to read 6 camera parameters"; return PTGPU_E_IO; }
    unsigned n = 0;
    if (std::fscanf(f, "size %u\n", &n) != 1) { std::fclose(f); err = "failed to read size"; return PTGPU_E_IO; }
    for (unsigned i = 0; i < n; ++i) {
        float r;
        ptgpu_vec cen, e, col;
        int mat = 0;
        int rc = std::fscanf(f, "sphere %f  %f %f %f  %f %f %f  %f %f %f  %d\n", &r, &cen.x, &cen.y,
                             &cen.z, &e.x, &e.y, &e.z, &col.x, &col.y, &col.z, &mat);
        if (rc != 11) { std::fclose(f); err = "failed to read sphere"; return PTGPU_E_IO; }
        int refl = mat == 1 ? PTGPU_SPEC : (mat == 2 ? PTGPU_REFR : PTGPU_DIFF);
        sc.shapes.push_back(sphere_shape(r, cen, e, col, refl));
    }
    std::fclose(f);
    sc.light_cnt = 0;     // ReadScene sets neither area nor lightCnt
    sc.walllight = true;
    return PTGPU_OK;
}

}  // namespace

int read_scene(const char *path, int width, int height, LoadedScene &out, std::string &err) {
    out = LoadedScene();
    if (!path) { err = "null path"; return PTGPU_E_INVAL; }
    const char *dot = std::strrchr(path, '.');
    if (!dot) { err = "scene file has no extension"; return PTGPU_E_INVAL; }
    const char *ext = dot + 1;
    if (!std::strcmp(ext, "txt")) return read_txt(path, width, height, out, err);
    if (!std::strcmp(ext, "scn")) return read_scn(path, width, height, out, err);
    if (!std::strcmp(ext, "ply")) { err = ".ply scenes are not supported"; return PTGPU_E_INVAL; }
    err = std::string("unknown scene extension .") + ext;
    return PTGPU_E_INVAL;
}

int read_scene_compact(const char *path, int width, int height, CompactScene &out, std::string &err) {
    out = CompactScene();
    if (!path) { err = "null path"; return PTGPU_E_INVAL; }
    const char *dot = std::strrchr(path, '.');
    if (!dot) { err = "scene file has no extension"; return PTGPU_E_INVAL; }
    const char *ext = dot + 1;
    if (!std::strcmp(ext, "txt")) {
        CompactSink sink(out);
        int st = parse_txt(path, width, height, out.camera, out.light_cnt, sink, err);
        out.walllight = false;
        return st;
    }
    if (!std::strcmp(ext, "scn")) {
        LoadedScene sc;
        int st = read_scn(path, width, height, sc, err);
        if (st != PTGPU_OK) return st;
        out.camera = sc.camera;
        out.light_cnt = sc.light_cnt;
        out.walllight = sc.walllight;
        if (!sc.shapes.empty()) {
            out.segs.emplace_back();
            out.segs.back().shapes = std::move(sc.shapes);
        }
        return PTGPU_OK;
    }
    if (!std::strcmp(ext, "ply")) { err = ".ply scenes are not supported"; return PTGPU_E_INVAL; }
    err = std::string("unknown scene extension .") + ext;
    return PTGPU_E_INVAL;
}

void add_wall_light(CompactScene &sc) {
    LoadedScene w;
    add_wall_light(w);
    if (sc.segs.empty() || sc.segs.back().model) sc.segs.emplace_back();
    std::vector<ptgpu_shape> &v = sc.segs.back().shapes;
    v.insert(v.end(), w.shapes.begin(), w.shapes.end());
}

ptgpu_shape model_shape(const SceneSegment &g, size_t t) {
    return model_triangle(g.obj, t, g.pos, g.scale, g.e, g.c, g.refl);
}

void add_wall_light(LoadedScene &sc) {     // smallptGPU.cpp:1448-1459
    const float R = 1e4f;
    auto v = [](float x, float y, float z) { ptgpu_vec r = {x, y, z}; return r; };
    const ptgpu_vec z = v(0.f, 0.f, 0.f);
    sc.shapes.push_back(sphere_shape(R, v(R + 25.0f, 0.0f, 0.0f), z, v(.75f, .25f, .25f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(R, v(-R - 25.0f, 0.0f, 0.0f), z, v(.25f, .25f, .75f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(R, v(0.0f, 0.0f, R - 25.0f), z, v(.75f, .75f, .75f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(R, v(0.0f, 0.0f, -R + 100.0f), z, v(0.f, 0.f, 0.f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(R, v(0.0f, R + 25.0f, 0.0f), z, v(.75f, .75f, .75f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(R, v(0.0f, -R - 25.0f, 0.0f), z, v(.75f, .75f, .75f), PTGPU_DIFF));
    sc.shapes.push_back(sphere_shape(5.0f, v(10.0f, -17.0f, 0.0f), z, v(.9f, .9f, .9f), PTGPU_SPEC));
    sc.shapes.push_back(sphere_shape(5.0f, v(-10.0f, -17.0f, 0.0f), z, v(.9f, .9f, .9f), PTGPU_REFR));
    sc.shapes.push_back(sphere_shape(2.f, v(10.0f, 15.0f, 0.0f), v(12.f, 12.f, 12.f), v(0.f, 0.f, 0.f), PTGPU_DIFF));
}

void update_camera(ptgpu_camera *cam) {
    float xd = sinf(cam->yaw) * cosf(cam->pitch);
    float yd = sinf(cam->pitch);
    float zd = cosf(cam->yaw) * cosf(cam->pitch);
    ptgpu_vec d = {-1.f * xd, -1.f * yd, -1.f * zd};
    auto norm = [](ptgpu_vec &v) {
        float l = 1.f / sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
        v.x = l * v.x; v.y = l * v.y; v.z = l * v.z;
    };
    norm(d);
    cam->dir = d;
    const ptgpu_vec up = {0.f, 1.f, 0.f};
    const float fov = (kPiF / 180.f) * 45.f;
    ptgpu_vec x = {d.y * up.z - d.z * up.y, d.z * up.x - d.x * up.z, d.x * up.y - d.y * up.x};
    norm(x);
    const float k = cam->width * fov / cam->height;
    x.x = k * x.x; x.y = k * x.y; x.z = k * x.z;
    cam->x = x;
    ptgpu_vec y = {x.y * d.z - x.z * d.y, x.z * d.x - x.x * d.z, x.x * d.y - x.y * d.x};
    norm(y);
    y.x = fov * y.x; y.y = fov * y.y; y.z = fov * y.z;
    cam->y = y;
}

void make_seeds(uint64_t master, uint32_t *seeds, uint32_t count) {
    uint64_t st = master;
    for (uint32_t i = 0; i < count; ++i) {
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        uint32_t v = (uint32_t)z;
        seeds[i] = v < 2u ? 2u : v;
    }
}

}  // namespace ptgpu
