/*
 * FriendsRender GB300 — C-ABI of the GPU SPPM render loop.
 *
 * Drop-in replacement for the per-iteration render loop of the reference's
 * Render::StochasticProgressivePhotonMapping (SPPM/SPPM/SPPM.h:15-189):
 * eye pass, photon pass, photon radius query and the N/tau/R update, run on
 * one GPU.  Plain C types only; every buffer argument is a host pointer
 * unless its name ends in _dev.  All calls return FR_OK (0) or an FR_ERR_*
 * code and set a thread-local message readable with fr_last_error().
 *
 * Threading: a context is used by one thread at a time; it owns one CUDA
 * stream.  Several contexts may coexist.
 */
#ifndef FRIENDSRENDER_H
#define FRIENDSRENDER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FR_OK = 0,
  FR_ERR_INVALID = 1,   /* bad argument or descriptor */
  FR_ERR_CUDA = 2,      /* CUDA runtime error */
  FR_ERR_OOM = 3,       /* device allocation failed */
  FR_ERR_DEVICE = 4,    /* a kernel reported an error (traversal stack) */
  FR_ERR_IO = 5         /* a scene or image file could not be read or decoded */
};

/* Surface types: the reference's Surface subclasses (SPPM/SPPM/material.h). */
enum {
  FR_MAT_DIFFUSE = 0,          /* DiffuseSurface  (material.h:163-177) */
  FR_MAT_METAL = 1,            /* MetalSurface    (material.h:396-425) */
  FR_MAT_GGX_CONDUCTOR = 2,    /* Roughconductor  (material.h:222-278) */
  FR_MAT_GGX_DIELECTRIC = 3,   /* GGXGlass        (material.h:280-394) */
  /* The demo's further surfaces (main.cpp:14-114). */
  FR_MAT_BIMETAL = 4,          /* BiMetalSurface          (material.h:427-463) */
  FR_MAT_GLASS = 5,            /* GlassSurface            (material.h:465-531) */
  FR_MAT_GLOSS_TRANSMIT = 6,   /* GlossTransmitSurface    (material.h:677-766) */
  FR_MAT_DIFFUSE_TRANSMIT = 7  /* DiffuseTransmitSurface  (material.h:637-675) */
};

enum { FR_CAMERA_PINHOLE = 0, FR_CAMERA_THINLENS = 1 };

/* Replaces the reference's SceneMaterialManager plug-in result
 * (SceneMaterial.h:13-16): an Attribute's Surface and SURFACE_PARAM
 * (material.h:35-90) plus its map_Kd / map_d / map_bump textures
 * (Scene.cpp:60-77).  Texture fields are indices into fr_scene_desc.textures
 * or -1. */
typedef struct fr_material_desc {
  int32_t type;            /* FR_MAT_* */
  int32_t sppm_surface;    /* SURFACE_PARAM::isSPPMSurface */
  int32_t opaque;          /* SURFACE_PARAM::IfOpeque */
  int32_t tex_albedo;      /* map_Kd: albedo, and emission of an emissive material */
  int32_t tex_roughness;   /* map_d: roughness = clamp(0.5*r, 0.05, 0.8) */
  int32_t tex_bump;        /* map_bump: normal map */
  float albedo[3];         /* Kd */
  float emission[3];       /* Ke; a material with Ke summing above 1e-5 makes its facets area lights */
  float index;             /* SURFACE_PARAM::Index */
  float roughness;         /* SURFACE_PARAM::Roughness */
  float extinction;        /* SURFACE_PARAM::Extinction */
  float reflectance;       /* SURFACE_PARAM::Reflectance */
} fr_material_desc;

/* RGBA8 texture, row j at texels + 4*width*j (stbi_load layout,
 * TextureUtility.cpp:12-35). */
typedef struct fr_texture_desc {
  int32_t width, height;
  const uint8_t* texels;
} fr_texture_desc;

/* Replaces Scene (Scene.h:55-93) as built by Scene::CreateScene
 * (Scene.cpp:13-218): per facet three corner positions, normals and UVs and
 * an attribute (material) index, in OBJ face order. */
typedef struct fr_scene_desc {
  int32_t num_facets;
  const float* positions;       /* num_facets * 9 */
  const float* normals;         /* num_facets * 9 */
  const float* uvs;             /* num_facets * 6 */
  const int32_t* material_ids;  /* num_facets */
  int32_t num_materials;
  const fr_material_desc* materials;
  int32_t num_textures;
  const fr_texture_desc* textures;
  /* Environment map lighting the eye paths that leave the scene (the
   * reference's IBL texture, LightSampler.cpp:22-26: texels converted to
   * 0.4 * c^2, SPHERE mapping IBL.h:96-104); NULL for none.  With one, an
   * eye path goes on after its hitpoint (SPPM.cpp:170-173) and a path that
   * misses adds the map's colour times its throughput to the pixel's direct
   * light (SPPM.cpp:290-300, 409-414), which the resolve adds
   * (SPPM.cpp:485). */
  const fr_texture_desc* environment;
} fr_scene_desc;

/* Replaces iCamera (Camera.h:11-54) with PinholeCamera / ThinLensCamera.
 * fov_degrees, focal_length and distance_to_lens are the constructor's Fov,
 * F and DistanceToLens; lens_width/height <= 0 keep the reference default
 * (the image-plane size, Camera.h:42-43). */
typedef struct fr_camera_desc {
  int32_t type;                 /* FR_CAMERA_* */
  int32_t width, height;        /* render target size */
  float position[3];
  float target[3];
  float fov_degrees;
  float focal_length;
  float distance_to_lens;
  float aspect;
  float lens_width, lens_height;
} fr_camera_desc;

enum {
  /* Drop the reference's stale photon slot (SPPM.cpp:672): off by default, so
   * the photon set of every iteration is the reference's. */
  FR_FLAG_FIX_STALE_PHOTON_SLOT = 1u,
  /* Resolve with the standard SPPM estimate (tau / (pi R^2 * all emitted
   * photons)) instead of the reference's, which divides by the emitted photons
   * times the pixel's NumGather / iterations (SPPM.cpp:485-488) and so changes
   * with the photon sampling.  Off by default (the reference's image); for
   * comparing sampling strategies such as the photon guide. */
  FR_FLAG_STANDARD_RESOLVE = 2u,
  /* End an eye or photon path where the sampled direction's BSDF value or pdf
   * is NaN or its pdf is zero.  The reference only ends paths with a BSDF
   * value below 1e-8 or a negative pdf (SPPM.cpp:278-281, 648-651) and goes
   * on with the others, whose hitpoints then carry a NaN or infinite weight
   * (its rough-dielectric BSDF returns NaN for a few rare directions), so a
   * pixel turns NaN once a photon lands at such a hitpoint.  Also ends a
   * photon path whose flux or PDF product is no longer finite (both grow
   * bounce by bounce; long paths among sharp rough dielectrics overflow both,
   * and their photons then carry inf / inf).  Off by default (the reference's
   * hitpoints and photons). */
  FR_FLAG_END_DEGENERATE_PATHS = 4u,
  /* Watertight ray-triangle test (Woop, Benthin and Wald, "Watertight
   * Ray/Triangle Intersection", JCGT 2(1), 2013) in place of the reference's
   * Moller-Trumbore (Intersect.cpp:67-89): a ray that crosses an edge or a
   * vertex shared by triangles of a closed mesh meets at least one of them,
   * where Moller-Trumbore's rounding can let it pass between them.  Same
   * acceptance rule (t > 1e-4, nearest t, equal t to the larger facet index)
   * and the same (u, v) meaning.  Off by default (the reference's test). */
  FR_FLAG_WATERTIGHT = 8u,
  /* Keep each pixel's accumulated photon count N (SharedHitPoint::NumPhoton,
   * SPPM.h:119) as a float.  The reference keeps an int, so N += M * alpha
   * truncates (SPPM.cpp:447) and the radius shrinks on a count that loses
   * up to one photon per update.  The per-pixel N that fr_read_state and the
   * checkpoint return then holds the float's bits.  Off by default (the
   * reference's count). */
  FR_FLAG_FLOAT_PHOTON_COUNT = 16u
};

typedef struct fr_sppm_params {
  int32_t photons_per_iteration;  /* the reference's NumPhotonsPerStep */
  float alpha;                    /* ppm_Alpha (SPPM.cpp:20), reference 0.9 */
  float initial_radius;           /* FirstRadius (SPPM.cpp:21), reference 0.015 */
  uint32_t flags;                 /* FR_FLAG_* */
  float grid_cell_scale;          /* photon grid cell = scale * mean hitpoint radius; <= 0 selects 2 */
  /* Learned photon-emission guide (no counterpart in the reference): photon
   * directions from a defensive mixture of cosine sampling and a network
   * trained online, with the mixture's pdf in the photon weight.  Iteration
   * k's photons train the network during iteration k + 1, so iteration k + 2
   * is the first to sample it.  Zero (guide = 0) is the reference's plain
   * emission. */
  int32_t guide;                  /* 1: guided emission */
  float guide_plain_fraction;     /* share of cosine sampling in the mixture; <= 0 selects 0.2 */
  int32_t guide_batch;            /* training samples per iteration; <= 0 selects 16384 */
  float guide_learning_rate;      /* Adam step size; <= 0 selects 0.005 */
  uint32_t guide_seed;            /* initial network weights */
  int32_t guide_steps;            /* Adam steps per iteration on its samples; <= 0 selects 16 (at most 64) */
  /* Scene BVH builder (no counterpart in the reference, which builds on the
   * host, bvh8.h:135-189): FR_BVH_HOST_SAH (0, binned SAH on the host) or
   * FR_BVH_DEVICE_LBVH (1, Morton-code radix tree built on the GPU).  Both
   * give the same hits; the SAH tree traces faster, the LBVH builds faster. */
  int32_t bvh_builder;
} fr_sppm_params;

enum { FR_BVH_HOST_SAH = 0, FR_BVH_DEVICE_LBVH = 1 };

typedef struct fr_stats {
  int64_t iterations;         /* iterations run so far */
  int64_t photon_paths;       /* photon paths emitted so far (TotalPhoton) */
  int64_t pixels;
  int64_t triangles;
  int64_t bvh_nodes;
  int64_t photon_table;       /* photon grid buckets */
  double device_bytes;        /* device memory held by the context */
} fr_stats;

typedef struct fr_ctx fr_ctx;

/* Message of the last failing call on this thread ("" if none). */
const char* fr_last_error(void);

/* Uploads the scene (building its BVH and light tables on the host), sets up
 * the camera and allocates all per-iteration buffers; nothing is allocated
 * later.  Replaces the set-up part of RenderImage_FixStep /
 * RenderImage_FixRenderTime (SPPM.cpp:682-766). */
int fr_create(const fr_scene_desc* scene, const fr_camera_desc* camera, const fr_sppm_params* params,
              fr_ctx** out);

/* ---------------------------------------------------------------- scene ingest
 * Scene::CreateScene (Scene.cpp:13-218) on the host, no GPU needed: reads an
 * OBJ file and its MTL libraries the way tinyobjloader 0.9.22 (vendored by the
 * reference as tiny_obj_loader.cpp) does with its default flags (polygons
 * fanned into triangles, vertices shared within a face group), decodes the
 * textures the MTL names, and returns an fr_scene_desc whose arrays the
 * fr_scene owns.
 *
 * asset_dir is the prefix put before MTL and texture names (the reference
 * hard-codes "meshData//", Scene.cpp:20-21; NULL means that).  MTL keys:
 * Kd albedo, Ke emission, map_Kd albedo texture, map_d roughness texture,
 * map_bump (or bump) normal map (Scene.cpp:60-77); a texture name of two
 * characters or fewer, or a file that does not decode, leaves that texture
 * unset, as in the reference.  A face whose usemtl names no material gets
 * material -1, which fr_create rejects (the reference's attribute lookup
 * throws on it).  environment_file, when not NULL, is decoded as the
 * environment map (the IBL texture main.cpp:132-143 hands to CreateScene).
 *
 * Images: PNG (all colour types, bit depths 1-16, Adam7) decoded to what
 * stb_image 2.12 returns with req_comp 0 (16-bit samples keep their high
 * byte; grey below 8 bits is scaled to 0..255; tRNS adds an alpha channel),
 * then widened to RGBA8 the way LoadTextureFromFile (TextureUtility.cpp:12-35)
 * fills a colour: C channels per pixel, C being the count stbi_load reports,
 * missing ones 0 and alpha 255 (so grey+alpha lands in red and green, and a
 * grey or RGB image with tRNS, whose reported C leaves out the added alpha,
 * is read with the reference's short stride).  Other formats return
 * FR_ERR_IO. */
typedef struct fr_scene fr_scene;

/* The material extension point, SceneMaterialManager::SetParamtoAttribute_p
 * (SceneMaterial.h:13-16): called once per MTL material, in file order, with
 * its name and a descriptor holding the Attribute's values before the call
 * (Scene.cpp:62-65): albedo = Kd, emission = Ke, index 1, roughness,
 * extinction and reflectance 1, opaque 1, sppm_surface 0, type
 * FR_MAT_DIFFUSE (SURFACE_PARAM(), material.h:76-89).  It may change any
 * field; the tex_* fields are set after it returns (Scene.cpp:72-76).  A
 * non-zero return fails the load with FR_ERR_INVALID.  A NULL callback keeps
 * the defaults, like the reference's default SceneMaterialManager (a diffuse
 * surface that is not an SPPM surface, so such a scene stores no hitpoints). */
typedef int (*fr_material_fn)(void* user, const char* material_name, fr_material_desc* material);

int fr_scene_load_obj(const char* obj_file, const char* asset_dir, const char* environment_file,
                      fr_material_fn material_fn, void* user, fr_scene** out);
/* The loaded scene, valid until fr_scene_free. */
const fr_scene_desc* fr_scene_get_desc(const fr_scene* scene);
/* Name of material m (newmtl), or NULL when m is out of range. */
const char* fr_scene_material_name(const fr_scene* scene, int32_t m);
void fr_scene_free(fr_scene* scene);

/* TextureUtility::LoadTextureFromFile (TextureUtility.cpp:12-35) for one
 * image file: writes its size and the channel count stb would report; when
 * rgba is not NULL, also width*height*4 bytes of RGBA8 (row j at
 * rgba + 4*width*j, the file's row order). */
int fr_texture_load(const char* file, int32_t* width, int32_t* height, int32_t* channels, uint8_t* rgba);

/* Enqueues n SPPM iterations (the loop body of RenderImage_FixRenderTime,
 * SPPM.cpp:768-848, with a fixed photon count).  Iteration k (counted from 1
 * over the context's life) uses the reference's seeds for step k.
 * Asynchronous; see fr_synchronize.  A context has three streams: the
 * photon pass and the photon grid run on the context's stream (fr_stream),
 * the eye pass and the gather on a pixel stream (an iteration's gather
 * overlaps the next iteration's photon pass), and a guided context's
 * training on a third.  Every other call on the context, and fr_stream
 * itself, first makes the context's stream wait for the other two, so work
 * queued on it after any of them sees every iteration enqueued so far. */
int fr_iterate(fr_ctx* ctx, int n);

/* Waits for the context's streams and reports kernel errors. */
int fr_synchronize(fr_ctx* ctx);

/* Batched rendering of uneven scenes (no counterpart in the reference, which
 * renders one scene per call): n iterations of each of `count` contexts,
 * iteration k of every context enqueued before iteration k + 1 of any.  Each
 * context replays its own iteration graph on its own streams, so the scenes'
 * kernels run concurrently and small scenes fill the SMs that large ones
 * leave idle.  Every context's results are those of fr_iterate.
 * Asynchronous; fr_synchronize each context. */
int fr_iterate_batch(fr_ctx* const* ctxs, int count, int n);

/* A batch graph (no counterpart in the reference): one CUDA graph holding one
 * iteration of every context of the batch, captured once by fr_batch_create,
 * so that fr_batch_iterate advances all the scenes with one graph launch per
 * iteration (fr_iterate_batch launches one graph per context).  The scenes'
 * iterations are independent branches of the graph and run concurrently.
 * Results are those of fr_iterate.  The batch keeps pointers to the
 * contexts: destroy it before them, and create it after fr_autotune (a
 * context's photon wavefront threshold is part of the captured graph).
 * fr_batch_iterate orders itself after the work already enqueued on each
 * context's stream and before the work enqueued there after it, so
 * fr_synchronize, fr_resolve and the other calls on a context see its
 * iterations; asynchronous like fr_iterate.  No context may have the stage
 * profiler on. */
typedef struct fr_batch fr_batch;
int fr_batch_create(fr_ctx* const* ctxs, int count, fr_batch** out);
int fr_batch_iterate(fr_batch* batch, int n);
void fr_batch_destroy(fr_batch* batch);

/* Autotuner (no counterpart in the reference): picks the context's photon
 * wavefront threshold (a round with fewer live paths hands them to the tail
 * kernel) from 4096, 8192, 16384, 32768 and 65536 by timing `iterations`
 * replays of the iteration graph with each (plus one untimed).  These are
 * real iterations of the render, 5 * (iterations + 1) in all; the threshold
 * changes the speed only, never a result.  *photon_tail_min (may be NULL)
 * receives the choice. */
int fr_autotune(fr_ctx* ctx, int iterations, uint32_t* photon_tail_min);

/* Writes the image (reconstructImageFromSharedPoints, SPPM.cpp:473-493):
 * width*height RGBA floats, pixel x + y*width.  rgba is a host pointer;
 * fr_resolve_dev takes a device pointer and does not synchronize. */
int fr_resolve(fr_ctx* ctx, float* rgba);
int fr_resolve_dev(fr_ctx* ctx, float* rgba_dev);

/* fr_resolve without the wait, so that the read-back overlaps the next
 * fr_iterate: queues the image of the current state and its copy into the
 * host buffer rgba (pinned memory lets the copy run alongside the next
 * iteration) on a copy stream of the context, and returns a ticket.  The
 * resolve runs on the pixel stream after the last gather, so the next
 * iteration's photon pass does not wait for it.
 * fr_resolve_wait(ticket) returns once that copy has landed; rgba must stay
 * valid until then.  The context holds two device images, used in turn, so
 * a third call's resolve waits on the device for the first call's copy.
 * Kernel errors are reported by the next fr_synchronize or fr_resolve. */
int fr_resolve_async(fr_ctx* ctx, float* rgba, uint64_t* ticket);
int fr_resolve_wait(fr_ctx* ctx, uint64_t ticket);

/* ExportPNG (TextureUtility.cpp:52-65): the current image resampled by the
 * reference's bilinear sampler at u = i / W, v = j / H and quantized to
 * max(0, min(255, int(c * 255))) per channel; width*height*4 bytes, row-major
 * RGBA into a caller-owned host buffer. */
int fr_resolve_rgba8(fr_ctx* ctx, uint8_t* rgba);

/* fr_resolve_rgba8 written as a PNG file (8-bit RGBA; the zlib stream holds
 * stored blocks, so the file differs from stb's but decodes to the same
 * pixels). */
int fr_export_png(fr_ctx* ctx, const char* path);

/* Writes width*height RGBA8 pixels as a PNG file; needs no GPU. */
int fr_write_png(const char* path, int32_t width, int32_t height, const uint8_t* rgba);

int fr_get_stats(fr_ctx* ctx, fr_stats* out);

/* The context's cudaStream_t (as void*), for callers that record events or
 * queue work on it; the stream first waits for the pixel stream (see
 * fr_iterate), so what follows on it sees every iteration enqueued so far. */
void* fr_stream(fr_ctx* ctx);

void fr_destroy(fr_ctx* ctx);

/* Stage profiler.  While enabled, fr_iterate records CUDA events around each
 * stage of an iteration and around each trace-round kernel (FR_STAGE_*), on
 * the stream the stage runs on (the eye pass and the gather run on the pixel
 * stream, so the eye and photon stages, and a gather and the next photon
 * stage, overlap in time); fr_profile_read synchronizes, returns the summed
 * milliseconds and the number of timed intervals per stage, then clears them.
 * max_iterations bounds the iterations profiled between reads (events are
 * created here).  *launches is the number of kernels fr_iterate has launched
 * so far. */
enum {
  FR_STAGE_EYE = 0,          /* eye pass (its own stream, concurrent with the photon pass) */
  FR_STAGE_PHOTON = 1,       /* photon pass */
  FR_STAGE_GRID = 2,         /* photon grid build */
  FR_STAGE_GATHER = 3,       /* gather and N/tau/R update */
  FR_STAGE_EYE_TRACE = 4,    /* the eye pass's trace-round kernels (inside FR_STAGE_EYE) */
  FR_STAGE_PHOTON_TRACE = 5, /* the photon pass's trace-round kernels (inside FR_STAGE_PHOTON) */
  FR_STAGES = 6
};
int fr_profile_enable(fr_ctx* ctx, int32_t on, int32_t max_iterations);
int fr_profile_read(fr_ctx* ctx, double* stage_ms, int64_t* stage_count, int64_t* launches);

/* ---------------------------------------------------------------- parity
 * Entry points the parity tests drive; each synchronizes before returning. */

/* Closest hit (Scene::GetOneFacetFromRay, Scene.cpp:224-237): rays are n x 7
 * floats {origin, direction, index}; MinT = 1e-4, MaxT = FLT_MAX.
 * facet[i] = -1 on a miss; tuv[i] = {t, u, v}. */
int fr_trace_closest(fr_ctx* ctx, const float* rays, int32_t n, int32_t* facet, float* tuv);

/* Any hit (findAnyElement, bvh8.h:643-707): rays are n x 8 floats
 * {origin, direction, min_t, max_t}; hit[i] = 1 if a triangle is met with
 * min_t < t <= max_t. */
int fr_trace_any(fr_ctx* ctx, const float* rays, int32_t n, int32_t* hit);

/* Radius query with the renderer's photon grid: for hitpoint h (position
 * hp[4h..4h+2], radius hp[4h+3]) counts photons p with
 * isIncludePoint(p, x - R, x + R) && |p - x|^2 < R^2 (kdtree.h:78-88,
 * SPPM.cpp:424-432).  If pairs is not NULL it receives up to pair_capacity
 * (hitpoint, photon) index pairs in any order and *pair_count the total.
 * A hitpoint whose radius is not finite or negative, or whose ball spans
 * more than 128 cells of `cell` along an axis, returns FR_ERR_INVALID. */
int fr_radius_query(fr_ctx* ctx, const float* hp, int32_t num_hitpoints, const float* photons_xyz,
                    int32_t num_photons, float cell, int32_t* counts, uint32_t* pairs, uint32_t pair_capacity,
                    uint32_t* pair_count);

/* Radius count that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot let the library call cudaMalloc: cudaMalloc and
 * cudaFree synchronize the whole device (stalling work on other streams),
 * and applications that hand out all device memory from their own pool at
 * start-up cannot have a library allocate on its own.  Same query as
 * fr_radius_query (counts only), with device pointers: hp_dev holds
 * num_hitpoints x {x, y, z, R} floats, photons_dev num_photons x {x, y, z}
 * floats, counts_dev receives num_hitpoints counts; the work is enqueued on
 * `stream` (a cudaStream_t, NULL for the default stream) and not waited for.
 * hp_dev must be 16-byte aligned (FR_ERR_INVALID otherwise), and the current
 * device must be the stream's device.  The grid's origin is 0: a hitpoint
 * whose radius is not finite, or whose ball spans more than 128 cells along
 * an axis or lies beyond 1e9 cells from the origin, gets the count -1 (the
 * host cannot check device inputs without waiting for them).
 * All intermediate buffers are fixed device arrays inside the library, sized
 * for FR_NOALLOC_MAX_PHOTONS photons (about 10.5 MB, held by every GPU that
 * loads the library until exit); more photons return FR_ERR_INVALID.  The
 * first call on a device looks up those arrays' device addresses: make it
 * before any stream capture.  Calls share the arrays (each call clears what
 * must start at zero), so calls that overlap on the GPU race. */
#define FR_NOALLOC_MAX_PHOTONS 262144
int fr_radius_count_noalloc(const float* hp_dev, int32_t num_hitpoints, const float* photons_dev,
                            int32_t num_photons, float cell, int32_t* counts_dev, void* stream);

/* No reference counterpart: a device self-check of the kernels' float
 * replacements for the reference's double-precision expressions.  Evaluates
 * each of FR_EXACT_FUNCTIONS functions on `samples` seeded random inputs both
 * ways and returns, per function, how often the float path produced a value
 * (fast_paths) and how often that value differed from the double expression's
 * (mismatches, 0 when the replacement is exact).  Functions, in order: pow_m2,
 * GGX sampling cos(theta), GGX sampling pdf, GGX glass cos(theta), GGX glass
 * refraction pdf, metal BRDF, conductor masking term, conductor tm3, conductor
 * square root. */
#define FR_EXACT_FUNCTIONS 9

/* No reference counterpart: a device self-check of the tensor-core (tcgen05)
 * GEMM the photon guide's network uses.  Multiplies seeded random BF16
 * matrices three ways (128x64x64, the same accumulated twice, and N = 48) and
 * returns the largest absolute error of each against a host GEMM on the same
 * inputs in max_abs_err[0..2]. */
int fr_check_tc_gemm(uint32_t seed, double* max_abs_err);
int fr_check_exact_math(uint64_t samples, uint32_t seed, uint64_t* mismatches, uint64_t* fast_paths);

/* The photon guide's state (contexts created with guide = 1).
 * fr_guide_params / fr_guide_set_params: the FP32 network parameters (the
 * training's latest; fr_guide_set_params also makes them the ones the next
 * emission samples)
 * (FR_GUIDE_PARAMS floats: W1[64][5], b1, W2[64][64], b2, W3[64][64], b3,
 * W4[48][64] (rows 40-47 zero), b4[48]).  fr_read_guide_importance: per photon
 * path, the flux its photons brought to hitpoints in the last iteration.
 * fr_guide_gradient: the gradient sums of the training loss
 * sum_j -I_j log q(d_j | x_j) over n samples (n x 9 floats: 5 inputs,
 * direction, importance I) computed by the training kernels, and sum_j I_j;
 * the network is not updated. */
#define FR_GUIDE_PARAMS 11824
int fr_guide_params(fr_ctx* ctx, float* params);
int fr_guide_set_params(fr_ctx* ctx, const float* params);
int fr_read_guide_importance(fr_ctx* ctx, float* importance);
int fr_guide_gradient(fr_ctx* ctx, int32_t n, const float* samples, float* grad, float* weight_sum);

/* No reference counterpart: the wavefront queue lengths of the last
 * iteration.  eye_counts[r] / photon_counts[r] is the number of paths traced
 * in round r (r < *eye_rounds / *photon_rounds; 0 for rounds skipped because
 * too few paths were left) and, at r = rounds, the number the tail kernel
 * finished; arrays of FR_MAX_WAVE_ROUNDS + 1 entries. */
#define FR_MAX_WAVE_ROUNDS 16
int fr_read_wave_counts(fr_ctx* ctx, uint32_t* eye_counts, uint32_t* photon_counts, int32_t* eye_rounds,
                        int32_t* photon_rounds);

/* Hitpoints of the last iteration (SoA, see HitpointBuf in the kernels):
 * each array width*height*4 floats; any pointer may be NULL. */
int fr_read_hitpoints(fr_ctx* ctx, float* pos_type, float* nrm_rough, float* out_mat, float* wgt_facet);

/* Photon slots after the last iteration: paths * 32 entries of 4 floats each
 * (pos+index, flux+pdf, dir+valid), path-major (path i's slot k at entry
 * i * 32 + k), and the per-path count of photons the compactor takes
 * (SPPM.cpp:812-822). */
int fr_read_photon_slots(fr_ctx* ctx, float* pos, float* flux, float* dir, uint32_t* counts);

/* Per-pixel photon count M and flux sum of the last iteration's gather. */
int fr_read_gather(fr_ctx* ctx, int32_t* m, float* phi4);

/* Direct (environment) light: the last iteration's per-pixel value
 * (HitPoint::DirectLight after the camera-pdf division, SPPM.cpp:345; 3
 * floats, zero where the path did not miss) and the per-pixel sums and counts
 * (SharedHitPoint::DirectLight / NumDirectLight).  Any pointer may be NULL. */
int fr_read_direct(fr_ctx* ctx, float* last3, float* sum3, int32_t* count);

/* Per-pixel progressive state: tau (3 doubles), N, R, NumGather. */
int fr_read_state(fr_ctx* ctx, double* tau, int32_t* n, float* r, int32_t* g);

/* The N/tau/R update of applyHitPointInfo (SPPM.cpp:444-449) alone: applies
 * per-pixel photon counts m (width*height) and flux sums phi (width*height*3)
 * to the context's state, with the arithmetic an iteration uses.  For
 * checking the update against the reference's own M and flux sums. */
int fr_update(fr_ctx* ctx, const int32_t* m, const float* phi);

/* fr_update with device-resident inputs: m_dev (width*height int32) and
 * phi4_dev (width*height x 4 floats, RGB and an unused fourth, 16-byte
 * aligned), applied on the context's stream without a host round trip.  For
 * a sharded render, where each GPU gathers its own photons and an all-reduce
 * of the per-pixel counts and flux sums precedes the update.  Asynchronous
 * (fr_synchronize). */
int fr_update_dev(fr_ctx* ctx, const int32_t* m_dev, const float* phi4_dev);

/* Checkpoint and resume between iterations (no counterpart in the reference,
 * which renders in one call).  fr_save_state with buf == NULL stores the
 * checkpoint size in *size; otherwise *size is buf's capacity on entry and
 * the bytes written on return.  The checkpoint holds the iteration count, the
 * per-pixel state and the photon slots; fr_load_state restores it into a
 * context created with the same scene, camera and parameters (checked:
 * resolution, photon paths, flags, alpha, initial radius, triangle count), after
 * which iterations continue exactly as they would have in the saved context.
 * A guided context's checkpoint also holds the network, its optimizer state
 * and the copy of the network the next emission samples.  Checkpoints of
 * another layout version (their first 8 bytes) are refused. */
int fr_save_state(fr_ctx* ctx, void* buf, size_t* size);
int fr_load_state(fr_ctx* ctx, const void* buf, size_t size);

/* Moves the random streams of a context on which no iteration has run: its
 * iteration k then draws the reference's seeds of step first_step + k instead
 * of step k (eye seed pixel + pixels * step, SPPM.cpp:334; photon seed
 * path + 135 + paths * step, SPPM.cpp:520; both 32-bit).  For independent
 * runs of one scene whose seed ranges do not overlap (a reference image,
 * replicas); the iteration count, the resolve and the checkpoint (which
 * carries first_step) are unchanged.  No counterpart in the reference. */
int fr_seek(fr_ctx* ctx, uint32_t first_step);

#ifdef __cplusplus
}
#endif

#endif /* FRIENDSRENDER_H */
