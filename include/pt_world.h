/*
 * pt_world.h - C ABI of the host-side world builder.
 *
 * Restates the parts of the reference's src/render/world.rs that produce the
 * GPU buffers the trace pass reads: the binned SAH BVH (Scene::subdivide,
 * world.rs:1430-1591) with the triangle reorder (world.rs:1339-1355), Vose
 * alias tables (world.rs:542-575), scene emissive uniforms and alias table
 * (world.rs:1691-1735), skybox normalisation, alias table and flux
 * (world.rs:1872-1987), light category probabilities (world.rs:484-498), the
 * auto camera and GpuCamera (world.rs:2159-2193), and World::take_updates
 * (world.rs:790-884).  Scenes come from a glTF file (ptw_load_gltf, with its
 * texture images packed into atlas layers), from meshes handed over in memory
 * (ptw_add_mesh) or from the procedural scene generators below; skyboxes from
 * .hdr / .exr files or pixels.
 *
 * All functions return PT_OK or an error code from pt.h; ptw_last_error
 * gives the message.
 */
#ifndef PT_WORLD_H
#define PT_WORLD_H

#include "pt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ptw_world ptw_world;

/* DEFAULT_SKYBOX_LUMINANCE, world.rs:21 */
#define PTW_DEFAULT_SKYBOX_LUMINANCE 8000.0f

/* A triangle mesh already in world space.  Optional arrays may be NULL:
 * normals -> flat normals per triangle (world.rs:1221-1235); uvs -> the
 * repeating (0,0),(1,0),(0,1) pattern (world.rs:1107-1111, 1170-1175);
 * tangents -> MikkTSpace frames per corner with the handedness negated, as
 * the reference computes them (world.rs:1238-1260); so are given tangents
 * that hold the (1, 0, 0, 1) placeholder or mix handedness within a
 * triangle (world.rs:1188-1217). */
typedef struct ptw_mesh {
    const float* positions;  /* vertex_count * 3 */
    const float* normals;    /* vertex_count * 3 or NULL */
    const float* uvs;        /* vertex_count * 2 or NULL */
    const float* tangents;   /* vertex_count * 4 or NULL */
    uint32_t vertex_count;
    const uint32_t* indices; /* index_count, a multiple of 3; NULL = 0..vertex_count */
    uint32_t index_count;
    uint32_t material_index;
} ptw_mesh;

int ptw_create(ptw_world** out);
void ptw_destroy(ptw_world* world);
const char* ptw_last_error(const ptw_world* world);

/* GpuMaterial::new defaults (world.rs:2041-2155) for a material with no
 * glTF fields set: base colour 1, metallic 1, roughness 1, ior 1.5, ... */
void ptw_default_material(pt_material* out);

int ptw_add_material(ptw_world* world, const pt_material* material, uint32_t* index);
int ptw_add_mesh(ptw_world* world, const ptw_mesh* mesh);
/* sRGB / linear RGBA8 atlas layers (PT_ATLAS_SIZE^2 * 4 bytes each); returns the layer index */
int ptw_add_atlas_layer(ptw_world* world, int srgb, const uint8_t* rgba8, int32_t* layer);

/* glTF 2.0 import (.glb, or .gltf with external or base64 buffers): adds the
 * default scene's triangle primitives and their materials, walking the node
 * tree as the reference's Scene::new does (world.rs:1078-1337; materials
 * world.rs:1992-2155).  Every image of the file (PNG or JPEG; buffer view,
 * data URI or file) is decoded as ptw_decode_texture_rgba8 does and packed
 * into new 8192^2 atlas layers, sRGB for images that a material uses as base
 * colour, emission or specular colour, linear otherwise (world.rs:893-1076);
 * material texture slots get the layer and the UV offset/scale of their
 * image.  Call before ptw_build.  On failure `error` (if given) receives the
 * reason. */
int ptw_load_gltf(ptw_world* world, const char* path, char* error, size_t error_size);
/* the same from a .glb (or self-contained .gltf) held in memory, as the
 * reference's Scene::new(bytes) takes it (world.rs:890); URIs that name
 * files cannot be resolved and fail */
int ptw_load_gltf_bytes(ptw_world* world, const void* bytes, size_t size, char* error, size_t error_size);

/* Builds the BVH over all added meshes, reorders triangles to BVH order and
 * sets the auto camera (the tail of Scene::new, world.rs:1339-1357).  Errors
 * with PT_ERR_INVALID_ARG if the scene has no triangles. */
int ptw_build(ptw_world* world);

/* Skybox::new on decoded pixels (world.rs:1872-1957): normalises to
 * solid-angle-weighted mean luminance 1; an all-black image becomes a black
 * 1x1 skybox.  Without a call the skybox is black. */
int ptw_set_skybox_rgba(ptw_world* world, const float* rgba, uint32_t width, uint32_t height);

/* Skybox::new on an image file (the reference decodes its skybox asset with
 * an image library, world.rs:1872-1880): Radiance RGBE (.hdr, "-Y H +X W"),
 * single-part scanline OpenEXR (HALF/FLOAT/UINT channels R, G, B [, A] or
 * Y; compression NONE, RLE, ZIPS, ZIP or PIZ), or a PNG / JPEG image (8- or
 * 16-bit samples divided by their maximum, as the library converts them),
 * chosen by the file's magic bytes.  On failure `error` (if given) receives the reason and the skybox is
 * unchanged. */
int ptw_set_skybox_file(ptw_world* world, const char* path, char* error, size_t error_size);
/* the same from an image held in memory, as World::replace_skybox(bytes)
 * takes it (world.rs:635-644) */
int ptw_set_skybox_bytes(ptw_world* world, const void* bytes, size_t size, char* error, size_t error_size);

/* Decodes the same image files to linear RGBA32F, row 0 at the top.  With
 * rgba == NULL only *width and *height are set; otherwise rgba must hold
 * capacity >= width * height * 4 floats (PT_ERR_OUT_OF_LIMITS if not). */
int ptw_read_image_rgba(const char* path, float* rgba, uint64_t capacity, uint32_t* width, uint32_t* height,
                        char* error, size_t error_size);

/* Decodes a glTF texture image (PNG, or baseline / extended / progressive
 * Huffman JPEG) held in memory to RGBA8 with the importer's format rules
 * (world.rs:949-1011): grey -> (l, l, l, 255), grey + alpha -> (l, a, 0, 255),
 * RGB -> (r, g, b, 255), 16-bit samples -> their high byte.  Images larger
 * than PT_ATLAS_SIZE on a side are refused.  With rgba == NULL only *width
 * and *height are set; otherwise rgba must hold width * height * 4 bytes. */
int ptw_decode_texture_rgba8(const void* bytes, size_t size, uint8_t* rgba, uint64_t capacity, uint32_t* width,
                             uint32_t* height, char* error, size_t error_size);

/* Saves an RGB8 image (width * height * 3 bytes, rows top to bottom) in the
 * format its extension names: .png, .jpg / .jpeg (baseline JPEG, quality
 * 75), .webp (lossless) or .ppm; the output formats of the reference's
 * `render --output` (headless.rs:30,118-126) plus PPM. */
int ptw_write_image(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height, char* error,
                    size_t error_size);

/* the procedural sky of the large scene (vertical gradient plus a Gaussian
 * sun lobe), width x height, passed through ptw_set_skybox_rgba */
int ptw_set_procedural_skybox(ptw_world* world, uint32_t width, uint32_t height);

/* World::edit_skybox_average_luminance (world.rs:646-648): clamped at 0 */
int ptw_edit_skybox_average_luminance(ptw_world* world, float luminance);

/* Camera::resize (world.rs:2261-2267) of the scene camera */
int ptw_set_aspect_ratio(ptw_world* world, float aspect_ratio);

/* World::edit_camera + Camera::translate_and_rotate_to / set_fov
 * (world.rs:708-716, 2270-2293).  NULL leaves a value unchanged; angles in
 * radians; pitch is clamped to [-pi/2, pi/2], fov to [0, pi). */
int ptw_edit_camera(ptw_world* world, const float* position3, const float* yaw,
                    const float* pitch, const float* fov);

/* World::edit_emission_scale (world.rs:655-692): every emissive material
 * (luminance of the emission colour times the emission weight above 0) gets
 * its emission strength at build time times max(scale, 0), overwriting edits
 * of that value; ptw_emission_scale returns the last scale (1 initially).
 * Only after ptw_build. */
int ptw_edit_emission_scale(ptw_world* world, float scale);
float ptw_emission_scale(const ptw_world* world);

/* World::edit_material (world.rs:735-787) restricted to replacing the
 * editable prefix (everything before alpha_mode) of one material */
int ptw_edit_material(ptw_world* world, uint32_t index, const pt_material* material);

/* World::take_updates (world.rs:790-884).  The pointers stored in *out and in
 * the scene/skybox upload structs it points to stay valid until the next
 * ptw_take_updates or ptw_destroy. */
int ptw_take_updates(ptw_world* world, pt_world_updates* out);

/* read access for tests and tools */
uint64_t ptw_triangle_count(const ptw_world* world);
uint64_t ptw_node_count(const ptw_world* world);
uint64_t ptw_material_count(const ptw_world* world);
const pt_triangle_geometry* ptw_geometries(const ptw_world* world);
const pt_triangle_attribute* ptw_attributes(const ptw_world* world);
const pt_bvh_node* ptw_bvh_nodes(const ptw_world* world);
const pt_material* ptw_materials(const ptw_world* world);
/* triangle order produced by the BVH build: bvh_order[i] = index of the
 * triangle before reordering that now sits at i */
const uint32_t* ptw_bvh_order(const ptw_world* world);
/* deepest deferred-stack use of the reference's traversal over this BVH
 * (checked against the 64-entry stack, trace.slang:632,786) */
uint32_t ptw_bvh_max_depth(const ptw_world* world);

/* ------------------------------------------------------------- utilities */

/* Vose's alias method, world.rs:542-575 (double weights in, entries out);
 * returns the number of entries written (0 when the weights sum to <= 0). */
uint64_t ptw_alias_table(const double* weights, uint64_t count, pt_skybox_alias_entry* out);

/* Binned SAH build on bare triangles (world.rs:1339-1345, 1430-1591):
 * writes at most 2 * count - 1 nodes and the triangle order; returns the
 * node count (0 for count == 0). */
uint64_t ptw_build_bvh(const pt_triangle_geometry* triangles, uint64_t count,
                       pt_bvh_node* nodes_out, uint32_t* order_out);

/* --------------------------------------------------- procedural scenes */

/* Cornell-box-style room of 36 triangles: 5 unit-room walls, two rotated
 * boxes 0.3 and 0.6 tall, a 0.25 x 0.25 emissive ceiling quad (radiance
 * 17, 12, 4), OpenPBR base-only diffuse materials, black skybox. */
int ptw_scene_cornell_box(ptw_world** out);

/* The same room as eight meshes (floor, ceiling, back, left, right, short
 * box, tall box, lamp) with procedural 1024 x 1024 RGBA8 base-colour
 * textures on four of them (floor and short box: checkers; back wall and
 * tall box: value noise), packed into one sRGB atlas layer: the precision
 * workload. */
int ptw_scene_cornell_box_textured(uint64_t seed, ptw_world** out);

typedef struct ptw_procedural_params {
    uint64_t seed;
    uint32_t grid_x, grid_z;       /* heightfield quads (2 triangles each) */
    uint32_t boxes;                /* 12 triangles each */
    uint32_t spheres;              /* icospheres */
    uint32_t sphere_subdivision;   /* 20 * 4^s triangles each */
    uint32_t emissive_triangles;   /* small emissive triangles added on top */
    uint32_t skybox_width, skybox_height; /* 0 = black skybox */
    float skybox_luminance;        /* average luminance after normalisation */
    int32_t textured;              /* 1: 1024^2 RGBA8 checker / noise base-colour textures on
                                      about half of the meshes (64 per sRGB atlas layer)   */
    int32_t non_opaque;            /* 1: about 10% of boxes and spheres ALPHA_MODE_BLEND
                                      with alpha in [0.3, 0.9]                              */
} ptw_procedural_params;

/* defaults of the large scene: 1024 x 512-quad heightfield with 4-octave
 * value noise, 2000 boxes, 200 icospheres of subdivision 4, 64 emissive
 * triangles with log-uniform radiance in [1, 100], 1024 x 512 sky */
void ptw_procedural_defaults(ptw_procedural_params* params);
int ptw_scene_procedural(const ptw_procedural_params* params, ptw_world** out);

#ifdef __cplusplus
}
#endif

#endif /* PT_WORLD_H */
