/*
 * ref_harness.cpp — drives WalkRay's own C++ sources (compiled unmodified
 * from the reference tree by oracle/Makefile into oracle/_ref/) on the
 * synthetic `.wrs` scenes.  Test infrastructure only: it produces the
 * reference answers that pin the C restatement (oracle/wr_oracle.c) and the
 * committed golden fixtures; nothing in the library links or runs it.
 *
 * Subcommands
 *   trace    scene.wrs rays.wrr out.bin [filter.bin]
 *            Scene::buildKDTree (scene.cpp:20-44) then KDTree::intersect
 *            (kdtree.cpp:349-353) per ray, OpenMP over rays.  With filter.bin
 *            (n x {i32 inside, i32 contact}) each ray is filtered by
 *            NoSelfCondition (noself.cpp:13-20) as in MCRenderer::samplePath.
 *            out: n x {u32 global tri id or 0xffffffff, f32 dist}
 *   dumptree scene.wrs out.bin
 *            the reference tree in depth-first pre-order:
 *            per node {u32 is_leaf, f32 min[3], f32 max[3], u32 ntri, u32 tris[ntri]}
 *   render   scene.wrs spp maxlen seed out.bin [nee|bpt|vcm radius|ppm radius]
 *            PathTracer::renderPixels (pathTracer.cpp:7-76) as it is: the
 *            per-spp tree rebuild and PFM write included; with `bpt`
 *            BidirectionalPathTracer::renderPixels (bidirPathTracer.cpp:10-56);
 *            with `vcm radius` VCMTracer::renderPixels (vcmTracer.cpp:6-92)
 *            with VCMTracer::setRadius(radius); with `ppm radius`
 *            PhotonMap::renderPixels (photonMap.cpp:20-148), setRadius(radius).  out: W*H*3 f32
 *            (row 0 = top, p = y*W + x).  Elapsed seconds on stderr.  With
 *            WR_REF_ELLIPSE_LOG=path a `ppm` render also writes the records of
 *            its anisotropic queries' ellipses there (see wrEllipseLog).
 */
#include "wr_ref_prelude.h"

#include <chrono>
#include <vector>
#include <unistd.h>
#include <omp.h>

#include "macros.h"
#include "rng.h"
#include "scene.h"
#include "abstractObj.h"
#include "mcRenderer.h"
#include "renderEngine.h"
#include "noself.h"
#include "diffuseObj.h"
#include "glossyObj.h"
#include "anisotropicGlossyObj.h"
#include "refractiveObj.h"
#include "reflectiveObj.h"
#include "emissiveObj.h"
#include "homogeneousVolume.h"
#include "HeterogeneousVolume.h"
// PathTracer keeps its NEE switch in the default-private section of a
// `class`; reading it as a struct makes the switch settable from here.
#define class struct
#include "pathTracer.h"
#undef class
#include "bidirPathTracer.h"
#include "vcmTracer.h"
#include "photonMap.h"

extern "C" {
#include "wrs_io.h"
}

using namespace LFJ;

namespace LFJ {
// renderEngine.cpp needs <io.h> and rapidxml (absent); its constructor and
// destructor are trivial (renderEngine.cpp:10-16, 93-101) and restated here.
RenderEngine::RenderEngine() {
    rng = new Rng(1234);
    scene.setRng(rng);
    renderer = NULL;
    config = NULL;
}
RenderEngine::~RenderEngine() {
    if (renderer) delete renderer;
}
}  // namespace LFJ

// Layout twin of KDTree::Node (kdtree.cpp:31-42), which is private to that
// file; used only to walk the finished tree for `dumptree`.
struct NodeTwin {
    NodeTwin* left;
    NodeTwin* right;
    std::vector<unsigned> triangleIndices;
    struct { vec3f minCoord, maxCoord; } boundingBox;
};
struct KDTreeTwin {  // KDTree's members in declaration order (kdtree.h:20-40)
    KDTree::Strategy strategy;
    NodeTwin* root;
};

static vec3f v3(const float* p) { return vec3f(p[0], p[1], p[2]); }

// The record hook of the anisotropic photon query (ref_shim/wr_ref_ellipse_log.h):
// with WR_REF_ELLIPSE_LOG=path, every call appends 22 f32 {kind, in_dir[3],
// aniso normal[3], reflected dir[3], hit normal[3], Nu, Nv, ratio, mX[3], mY[3]}.
void wrEllipseLog(int kind, float ix, float iy, float iz, float nx, float ny, float nz, float sx, float sy, float sz,
                  float hx, float hy, float hz, float nu, float nv, float ratio, float ex, float ey, float ez,
                  float fx, float fy, float fz) {
    static FILE* out = NULL;
    static bool opened = false;
    const float rec[22] = {(float)kind, ix, iy, iz, nx, ny, nz, sx, sy, sz, hx, hy, hz,
                           nu, nv, ratio, ex, ey, ez, fx, fy, fz};
#pragma omp critical(wr_ellipse_log)
    {
        if (!opened) {
            opened = true;
            const char* path = getenv("WR_REF_ELLIPSE_LOG");
            out = path ? fopen(path, "wb") : NULL;
        }
        if (out) fwrite(rec, sizeof rec, 1, out);
    }
}

static void build_scene(RenderEngine& eng, const wrs_scene& ws, Rng* rng) {
    Scene& sc = eng.scene;
    for (uint32_t oi = 0; oi < ws.num_objects; oi++) {
        const wr_object_desc& d = ws.objects[oi];
        AbstractObject* obj = NULL;
        // HeterogeneousVolume captures scene->objects.size() as its id in the
        // constructor, so each object is created right before it is added.
        switch (d.type) {
            case WR_MAT_DIFFUSE: obj = new DiffuseObject(&sc); break;
            case WR_MAT_GLOSSY: obj = new GlossyObject(&sc); break;
            case WR_MAT_ANISO: obj = new AnisotropicGlossyObject(&sc); break;
            case WR_MAT_REFRACTIVE: obj = new RefractiveObject(&sc); break;
            case WR_MAT_EMISSIVE: obj = new EmissiveObject(&sc); break;
            case WR_MAT_HOMOGENEOUS: obj = new HomogeneousVolume(&sc, d.g); break;
            case WR_MAT_HETEROGENEOUS: obj = new HeterogeneousVolume(&sc, d.g); break;
            case WR_MAT_REFLECTIVE: obj = new ReflectiveObject(&sc); break;
            default: fprintf(stderr, "unknown object type %u\n", d.type); exit(2);
        }
        obj->setRng(rng);
        for (uint32_t v = 0; v < d.vert_count; v++) obj->vertexList.push_back(v3(ws.vertices + 3 * (d.vert_begin + v)));
        for (uint32_t t = 0; t < d.tri_count; t++) {
            const uint32_t* tri = ws.triangles + 3 * (d.tri_begin + t);
            obj->faceVertexIndexList.push_back(vec3ui(tri[0], tri[1], tri[2]));
        }
        obj->getBoundingBox(obj->minCoord, obj->maxCoord);
        vec3f a = v3(d.albedo), e = v3(d.emission);
        switch (d.type) {
            case WR_MAT_DIFFUSE: static_cast<DiffuseObject*>(obj)->setColor(a); break;
            case WR_MAT_GLOSSY:
                static_cast<GlossyObject*>(obj)->setColor(a);
                static_cast<GlossyObject*>(obj)->setPower(d.power);
                break;
            case WR_MAT_ANISO:
                static_cast<AnisotropicGlossyObject*>(obj)->setRs_Rd_Nu_Nv(v3(d.rs), v3(d.rd), d.nu, d.nv);
                break;
            case WR_MAT_REFRACTIVE:
                static_cast<RefractiveObject*>(obj)->setIOR(d.ior);
                static_cast<RefractiveObject*>(obj)->setDecayColor(v3(d.decay));
                break;
            case WR_MAT_EMISSIVE: static_cast<EmissiveObject*>(obj)->setColor(e); break;
            case WR_MAT_REFLECTIVE: static_cast<ReflectiveObject*>(obj)->setColor(a); break;
            case WR_MAT_HOMOGENEOUS:
                static_cast<HomogeneousVolume*>(obj)->setSigma(v3(d.sigma_s), v3(d.sigma_a));
                static_cast<HomogeneousVolume*>(obj)->setIOR(d.ior);
                // the ray-marching step of PhotonMap's volume estimate; the
                // constructor leaves it unset (homogeneousVolume.h:11, 76-81)
                static_cast<HomogeneousVolume*>(obj)->setStepSize(d.step_size);
                break;
            case WR_MAT_HETEROGENEOUS: {
                HeterogeneousVolume* hv = static_cast<HeterogeneousVolume*>(obj);
                hv->setSigma(v3(d.sigma_s), v3(d.sigma_a));
                hv->setIOR(d.ior);
                hv->setDensityScale(d.density_scale);
                hv->setStepSize(d.step_size);
                const wr_grid_desc& g = ws.grids[d.grid_index];
                // the reference reads its grid from a whitespace-separated text file
                char path[256];
                snprintf(path, sizeof path, "wr_ref_grid_%d_%u.txt", (int)getpid(), oi);
                FILE* f = fopen(path, "w");
                fprintf(f, "%u %u %u\n", g.nx, g.ny, g.nz);
                size_t cnt = (size_t)g.nx * g.ny * g.nz;
                for (size_t i = 0; i < cnt; i++) fprintf(f, "%.9g\n", g.density[i]);
                fclose(f);
                hv->loadDensityMap(path);
                unlink(path);
                break;
            }
        }
        sc.objects.push_back(obj);
    }
    const wr_camera_desc& c = ws.camera;
    sc.mCamera.setup(v3(c.position), v3(c.focus), v3(c.up), vec2f((float)c.width, (float)c.height),
                     c.image_plane_dist, rng);
    if (c.lens_radius > 0.f) sc.mCamera.setDOFParameters(c.lens_radius, c.focal_dist);
    sc.name = "wr";
}

static int cmd_trace(int argc, char** argv) {
    if (argc < 5) return 2;
    wrs_scene ws;
    if (wrs_load(argv[2], &ws)) { fprintf(stderr, "cannot read %s\n", argv[2]); return 1; }
    uint64_t n = 0;
    float* rays = wrs_load_rays(argv[3], &n);
    if (!rays) { fprintf(stderr, "cannot read %s\n", argv[3]); return 1; }
    std::vector<int32_t> filt;
    if (argc > 5) {
        filt.resize(2 * n);
        FILE* f = fopen(argv[5], "rb");
        if (!f || fread(filt.data(), 8, n, f) != n) { fprintf(stderr, "bad filter file\n"); return 1; }
        fclose(f);
    }
    RenderEngine* eng = new RenderEngine();
    build_scene(*eng, ws, eng->rng);
    auto t0 = std::chrono::steady_clock::now();
    eng->scene.buildKDTree(true);
    auto t1 = std::chrono::steady_clock::now();
    std::vector<uint32_t> out(2 * n);
    Scene& sc = eng->scene;
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        KDTree::Ray r;
        r.origin = v3(rays + 6 * i);
        r.direction = v3(rays + 6 * i + 3);
        unsigned tid = 0xffffffffu;
        float dist;
        if (filt.empty()) {
            dist = sc.tree.intersect(r, tid, NULL);
        } else {
            Ray pr;
            pr.origin = r.origin;
            pr.direction = r.direction;
            pr.insideObj = filt[2 * i] >= 0 ? sc.objects[filt[2 * i]] : NULL;
            pr.contactObj = filt[2 * i + 1] >= 0 ? sc.objects[filt[2 * i + 1]] : NULL;
            NoSelfCondition cond(&sc, pr);
            dist = sc.tree.intersect(r, tid, &cond);
        }
        out[2 * i] = dist >= 0 ? tid : 0xffffffffu;
        memcpy(&out[2 * i + 1], &dist, 4);
    }
    auto t2 = std::chrono::steady_clock::now();
    FILE* f = fopen(argv[4], "wb");
    fwrite(out.data(), 4, 2 * n, f);
    fclose(f);
    fprintf(stderr, "build_s %.3f trace_s %.3f threads %d\n", std::chrono::duration<double>(t1 - t0).count(),
            std::chrono::duration<double>(t2 - t1).count(), omp_get_max_threads());
    return 0;
}

static void dump_node(FILE* f, const NodeTwin* n) {
    uint32_t leaf = (n->left == NULL && n->right == NULL) ? 1u : 0u;
    fwrite(&leaf, 4, 1, f);
    fwrite(&n->boundingBox.minCoord.x, 4, 3, f);
    fwrite(&n->boundingBox.maxCoord.x, 4, 3, f);
    uint32_t cnt = leaf ? (uint32_t)n->triangleIndices.size() : 0u;
    fwrite(&cnt, 4, 1, f);
    if (cnt) fwrite(n->triangleIndices.data(), 4, cnt, f);
    if (!leaf) {
        dump_node(f, n->left);
        dump_node(f, n->right);
    }
}

static int cmd_dumptree(int argc, char** argv) {
    if (argc < 4) return 2;
    wrs_scene ws;
    if (wrs_load(argv[2], &ws)) return 1;
    RenderEngine* eng = new RenderEngine();
    build_scene(*eng, ws, eng->rng);
    eng->scene.buildKDTree(true);
    const KDTreeTwin* twin = reinterpret_cast<const KDTreeTwin*>(&eng->scene.tree);
    FILE* f = fopen(argv[3], "wb");
    dump_node(f, twin->root);
    fclose(f);
    return 0;
}

static int cmd_render(int argc, char** argv) {
    if (argc < 7) return 2;
    wrs_scene ws;
    if (wrs_load(argv[2], &ws)) return 1;
    unsigned spp = (unsigned)atoi(argv[3]), maxlen = (unsigned)atoi(argv[4]);
    int seed = atoi(argv[5]);
    bool nee = argc > 7 && strcmp(argv[7], "nee") == 0;
    bool bpt = argc > 7 && strcmp(argv[7], "bpt") == 0;
    bool vcm = argc > 8 && strcmp(argv[7], "vcm") == 0;
    bool ppm = argc > 8 && strcmp(argv[7], "ppm") == 0;
    RenderEngine* eng = new RenderEngine();
    delete eng->rng;
    eng->rng = new Rng(seed);
    eng->scene.setRng(eng->rng);
    build_scene(*eng, ws, eng->rng);
    // Config::load builds the global tree, RenderEngine::renderFilm the
    // per-object trees (config.cpp:519, renderEngine.cpp:27-30)
    eng->scene.buildKDTree(true);
    eng->scene.buildObjKDTrees(true);
    MCRenderer* pt;
    if (bpt) {
        pt = new BidirectionalPathTracer(eng, spp, maxlen);
    } else if (ppm) {
        PhotonMap* m = new PhotonMap(eng, spp, maxlen);
        m->setRadius((float)atof(argv[8]));
        pt = m;
    } else if (vcm) {
        VCMTracer* v = new VCMTracer(eng, spp, maxlen);
        v->setRadius((float)atof(argv[8]));
        pt = v;
    } else {
        PathTracer* p = new PathTracer(eng, spp, maxlen);
        p->name = "PathTracer";
        p->useNextEventEstimation = nee;
        pt = p;
    }
    eng->renderer = pt;
    const char* wd = getenv("WR_REF_WORKDIR");
    if (chdir(wd ? wd : "/tmp") != 0) return 1;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<vec3f> img = pt->renderPixels();
    auto t1 = std::chrono::steady_clock::now();
    FILE* f = fopen(argv[6], "wb");
    if (!f) return 1;
    fwrite(&img[0].x, 4, 3 * img.size(), f);
    fclose(f);
    fprintf(stderr, "render_s %.3f paths %llu threads %d\n", std::chrono::duration<double>(t1 - t0).count(),
            (unsigned long long)img.size() * spp, omp_get_max_threads());
    return 0;
}

// mesh file single|group out.bin [16 floats, row-major transform]: meshes as
// WalkRay loads them for Config::load (config.cpp:456-507, mesh.cpp:5-158).
// single: Mesh::loadShape(file) (unitized), world positions through the
// transform; group: the GroupObject flow (transform on the whole mesh, then
// loadShape(file, true, &shapes)), each shape's world positions.  Output per
// mesh: name length + name, vertex count + x y z floats, face count + indices.
static int cmd_mesh(int argc, char** argv) {
    if (argc < 5) return 2;
    float v[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    for (int k = 0; k < 16 && 5 + k < argc; k++) v[k] = (float)atof(argv[5 + k]);
    mat4f T;
    T.set_value(v);  // readMatrix: set_value, then transpose (config.cpp:610-619)
    T = transpose(T);
    std::vector<Mesh*> meshes;
    Mesh single, group;
    std::vector<Mesh*> shapes;
    if (!strcmp(argv[3], "single")) {
        single.loadShape(argv[2]);
        single.setTransform(T);
        meshes.push_back(&single);
    } else {
        group.setTransform(T);
        group.loadShape(argv[2], true, &shapes);
        meshes = shapes;
    }
    FILE* f = fopen(argv[4], "wb");
    if (!f) return 1;
    const uint32_t n = (uint32_t)meshes.size();
    fwrite(&n, 4, 1, f);
    for (Mesh* m : meshes) {
        const uint32_t len = (uint32_t)m->name.size();
        fwrite(&len, 4, 1, f);
        fwrite(m->name.data(), 1, len, f);
        const uint32_t nv = m->getVertexNum(), nf = m->getTriangleNum();
        fwrite(&nv, 4, 1, f);
        for (uint32_t i = 0; i < nv; i++) {
            vec3f w = m->getWorldVertexPosition(i);
            fwrite(&w.x, 4, 3, f);
        }
        fwrite(&nf, 4, 1, f);
        for (uint32_t i = 0; i < nf; i++) {
            vec3ui t = m->getVertexIndices(i);
            uint32_t t3[3] = {t.x, t.y, t.z};
            fwrite(t3, 4, 3, f);
        }
    }
    fclose(f);
    for (Mesh* s : shapes) delete s;
    return 0;
}

#ifdef WR_DROPIN
#include "gpuPathTracer.h"
// describe scene.wrs out.bin: the drop-in renderer's reading of every
// object's material (wrDefaultDescribe), as wr_object_desc records; objects
// it cannot describe get type 0xffffffff
static int cmd_describe(int argc, char** argv) {
    if (argc < 4) return 2;
    wrs_scene ws;
    if (wrs_load(argv[2], &ws)) return 1;
    RenderEngine* eng = new RenderEngine();
    build_scene(*eng, ws, eng->rng);
    FILE* f = fopen(argv[3], "wb");
    for (AbstractObject* o : eng->scene.objects) {
        wr_object_desc d;
        memset(&d, 0, sizeof d);
        if (!wrDefaultDescribe(o, &d)) d.type = 0xffffffffu;
        fwrite(&d, sizeof d, 1, f);
    }
    fclose(f);
    return 0;
}
#endif

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: wr_ref trace|dumptree|render ...\n");
        return 2;
    }
    std::ios::sync_with_stdio(true);
    std::cout.setstate(std::ios::failbit);  // the reference logs to stdout freely
    if (!strcmp(argv[1], "trace")) return cmd_trace(argc, argv);
    if (!strcmp(argv[1], "dumptree")) return cmd_dumptree(argc, argv);
    if (!strcmp(argv[1], "render")) return cmd_render(argc, argv);
    if (!strcmp(argv[1], "mesh")) return cmd_mesh(argc, argv);
#ifdef WR_DROPIN
    if (!strcmp(argv[1], "describe")) return cmd_describe(argc, argv);
#endif
    fprintf(stderr, "unknown command %s\n", argv[1]);
    return 2;
}
