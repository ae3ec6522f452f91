/*
 * wr_oracle_main.c — command-line front end of the C restatement (test
 * infrastructure only), mirroring oracle/ref_harness.cpp so that outputs of
 * the two can be compared byte for byte:
 *   wr_oracle trace    scene.wrs rays.wrr out.bin [filter.bin]
 *   wr_oracle dumptree scene.wrs out.bin
 *   wr_oracle render   scene.wrs spp maxlen seed out.bin [nee]
 *   wr_oracle count    scene.wrs rays.wrr      (AABB / triangle tests per ray)
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "wr_oracle.h"
#include "wrs_io.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void to_desc(const wrs_scene* ws, wr_scene_desc* d) {
    memset(d, 0, sizeof *d);
    d->num_objects = ws->num_objects;
    d->num_vertices = ws->num_vertices;
    d->num_triangles = ws->num_triangles;
    d->num_grids = ws->num_grids;
    d->objects = ws->objects;
    d->vertices = ws->vertices;
    d->triangles = ws->triangles;
    d->grids = ws->grids;
    d->camera = ws->camera;
}

static uint32_t* global_tris(const wrs_scene* ws, int32_t** tri_obj) {
    uint32_t* g = (uint32_t*)malloc(sizeof(uint32_t) * 3 * ((size_t)ws->num_triangles + 1));
    *tri_obj = (int32_t*)malloc(sizeof(int32_t) * ((size_t)ws->num_triangles + 1));
    for (uint32_t o = 0; o < ws->num_objects; o++) {
        const wr_object_desc* m = &ws->objects[o];
        for (uint32_t t = 0; t < m->tri_count; t++) {
            size_t gi = (size_t)m->tri_begin + t;
            for (int k = 0; k < 3; k++) g[3 * gi + k] = ws->triangles[3 * gi + k] + m->vert_begin;
            (*tri_obj)[gi] = (int32_t)o;
        }
    }
    return g;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: wr_oracle trace|dumptree|render|count ...\n");
        return 2;
    }
    wrs_scene ws;
    if (wrs_load(argv[2], &ws)) {
        fprintf(stderr, "cannot read %s\n", argv[2]);
        return 1;
    }
    if (!strcmp(argv[1], "trace") || !strcmp(argv[1], "count")) {
        uint64_t n = 0;
        float* rays = wrs_load_rays(argv[3], &n);
        if (!rays) return 1;
        int32_t* tri_obj;
        uint32_t* g = global_tris(&ws, &tri_obj);
        double t0 = now_s();
        wro_tree* T = wro_build(ws.vertices, ws.num_vertices, g, ws.num_triangles);
        double t1 = now_s();
        int32_t *inside = NULL, *contact = NULL;
        if (argc > 5) {
            int32_t* f = (int32_t*)malloc(8 * n);
            FILE* fh = fopen(argv[5], "rb");
            if (!fh || fread(f, 8, n, fh) != n) return 1;
            fclose(fh);
            inside = (int32_t*)malloc(4 * n);
            contact = (int32_t*)malloc(4 * n);
            for (uint64_t i = 0; i < n; i++) {
                inside[i] = f[2 * i];
                contact[i] = f[2 * i + 1];
            }
        }
        uint32_t* tri = (uint32_t*)malloc(4 * n);
        float* t = (float*)malloc(4 * n);
        uint64_t nb = 0, nt = 0;
        wro_trace(T, rays, n, inside, contact, tri_obj, tri, t, 0, &nb, &nt);
        double t2 = now_s();
        if (!strcmp(argv[1], "count")) {
            printf("{\"rays\": %llu, \"box_tests_per_ray\": %.4f, \"tri_tests_per_ray\": %.4f, \"nodes\": %u}\n",
                   (unsigned long long)n, (double)nb / n, (double)nt / n, wro_tree_num_nodes(T));
            return 0;
        }
        FILE* f = fopen(argv[4], "wb");
        for (uint64_t i = 0; i < n; i++) {
            fwrite(&tri[i], 4, 1, f);
            fwrite(&t[i], 4, 1, f);
        }
        fclose(f);
        fprintf(stderr, "build_s %.3f trace_s %.3f\n", t1 - t0, t2 - t1);
        return 0;
    }
    if (!strcmp(argv[1], "dumptree")) {
        int32_t* tri_obj;
        uint32_t* g = global_tris(&ws, &tri_obj);
        wro_tree* T = wro_build(ws.vertices, ws.num_vertices, g, ws.num_triangles);
        uint64_t need = wro_tree_dump(T, NULL, 0);
        void* buf = malloc(need + 1);
        wro_tree_dump(T, buf, need);
        FILE* f = fopen(argv[3], "wb");
        fwrite(buf, 1, need, f);
        fclose(f);
        return 0;
    }
    if (!strcmp(argv[1], "render") && argc >= 7) {
        wr_scene_desc d;
        to_desc(&ws, &d);
        uint32_t spp = (uint32_t)atoi(argv[3]), maxlen = (uint32_t)atoi(argv[4]);
        uint64_t seed = strtoull(argv[5], NULL, 10);
        uint32_t flags = (argc > 7 && !strcmp(argv[7], "nee")) ? WRO_NEE : 0;
        wro_scene* s = wro_scene_create(&d);
        uint32_t np = ws.camera.width * ws.camera.height;
        double* sum = (double*)calloc(3 * (size_t)np, sizeof(double));
        double t0 = now_s();
        uint64_t rays = 0;
        wro_render(s, maxlen, seed, flags, 0, np, 0, spp, sum, NULL, 0, &rays);
        double t1 = now_s();
        float* img = (float*)malloc(sizeof(float) * 3 * np);
        for (size_t i = 0; i < 3 * (size_t)np; i++) img[i] = (float)(sum[i] / spp);
        FILE* f = fopen(argv[6], "wb");
        fwrite(img, 4, 3 * (size_t)np, f);
        fclose(f);
        fprintf(stderr, "render_s %.3f paths %llu rays %llu\n", t1 - t0, (unsigned long long)np * spp,
                (unsigned long long)rays);
        return 0;
    }
    fprintf(stderr, "unknown command %s\n", argv[1]);
    return 2;
}
