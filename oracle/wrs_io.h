/*
 * wrs_io.h — reader for the `.wrs` scene files written by
 * walkray_gb300/scenes.py (Scene.save) and the `.wrr` ray files
 * (scenes.save_rays).  Test infrastructure only: used by the oracle
 * programs (the C restatement and the reference harness), never by the
 * library.  Plain C99, header-only.
 *
 * .wrs layout (little endian):
 *   "WRS1" u32 version u32 num_objects u32 num_vertices u32 num_triangles u32 num_grids
 *   camera: f32 position[3] focus[3] up[3]; u32 width height; f32 image_plane_dist lens_radius focal_dist
 *   wr_object_desc[num_objects]; f32 vertices[nv*3]; u32 triangles[nt*3] (object-local indices)
 *   per grid: u32 nx ny nz; f32 p0[3] p1[3]; f32 density[nx*ny*nz]
 */
#ifndef WRS_IO_H
#define WRS_IO_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/walkray.h"

typedef struct wrs_scene {
    uint32_t num_objects, num_vertices, num_triangles, num_grids;
    wr_object_desc* objects;
    float* vertices;
    uint32_t* triangles;
    wr_grid_desc* grids;
    wr_camera_desc camera;
} wrs_scene;

static int wrs__read(FILE* f, void* p, size_t n) { return fread(p, 1, n, f) == n ? 0 : -1; }

static int wrs_load(const char* path, wrs_scene* s) {
    memset(s, 0, sizeof(*s));
    FILE* f = fopen(path, "rb");
    if (!f) return -1;
    char magic[4];
    uint32_t hdr[5];
    int rc = wrs__read(f, magic, 4) || memcmp(magic, "WRS1", 4) || wrs__read(f, hdr, sizeof hdr);
    if (rc) { fclose(f); return -1; }
    s->num_objects = hdr[1]; s->num_vertices = hdr[2]; s->num_triangles = hdr[3]; s->num_grids = hdr[4];
    float cam9[9]; uint32_t wh[2]; float c3[3];
    rc |= wrs__read(f, cam9, sizeof cam9) || wrs__read(f, wh, sizeof wh) || wrs__read(f, c3, sizeof c3);
    memcpy(s->camera.position, cam9, 12); memcpy(s->camera.focus, cam9 + 3, 12); memcpy(s->camera.up, cam9 + 6, 12);
    s->camera.width = wh[0]; s->camera.height = wh[1];
    s->camera.image_plane_dist = c3[0]; s->camera.lens_radius = c3[1]; s->camera.focal_dist = c3[2];
    s->objects = (wr_object_desc*)malloc(sizeof(wr_object_desc) * (s->num_objects + 1));
    s->vertices = (float*)malloc(sizeof(float) * 3 * ((size_t)s->num_vertices + 1));
    s->triangles = (uint32_t*)malloc(sizeof(uint32_t) * 3 * ((size_t)s->num_triangles + 1));
    s->grids = (wr_grid_desc*)calloc(s->num_grids + 1, sizeof(wr_grid_desc));
    rc |= wrs__read(f, s->objects, sizeof(wr_object_desc) * s->num_objects);
    rc |= wrs__read(f, s->vertices, sizeof(float) * 3 * (size_t)s->num_vertices);
    rc |= wrs__read(f, s->triangles, sizeof(uint32_t) * 3 * (size_t)s->num_triangles);
    for (uint32_t g = 0; g < s->num_grids && !rc; g++) {
        uint32_t n3[3]; float p[6];
        rc |= wrs__read(f, n3, sizeof n3) || wrs__read(f, p, sizeof p);
        wr_grid_desc* gd = &s->grids[g];
        gd->nx = n3[0]; gd->ny = n3[1]; gd->nz = n3[2];
        memcpy(gd->p0, p, 12); memcpy(gd->p1, p + 3, 12);
        size_t cnt = (size_t)gd->nx * gd->ny * gd->nz;
        float* d = (float*)malloc(sizeof(float) * (cnt + 1));
        rc |= wrs__read(f, d, sizeof(float) * cnt);
        gd->density = d;
    }
    fclose(f);
    return rc ? -1 : 0;
}

static void wrs_free(wrs_scene* s) {
    for (uint32_t g = 0; g < s->num_grids; g++) free((void*)s->grids[g].density);
    free(s->objects); free(s->vertices); free(s->triangles); free(s->grids);
    memset(s, 0, sizeof(*s));
}

/* rays: returns malloc'd n x 6 floats */
static float* wrs_load_rays(const char* path, uint64_t* n) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    char magic[4];
    if (wrs__read(f, magic, 4) || memcmp(magic, "WRR1", 4) || wrs__read(f, n, 8)) { fclose(f); return NULL; }
    float* r = (float*)malloc(sizeof(float) * 6 * (*n + 1));
    if (wrs__read(f, r, sizeof(float) * 6 * *n)) { free(r); fclose(f); return NULL; }
    fclose(f);
    return r;
}

#endif
