//! pt_ffi.rs - Rust binding of the GB300 trace pass (include/pt.h) for the
//! reference renderer, replacing its wgpu `PathTracer`
//! (src/render/path_tracer.rs) in the headless renderer
//! (src/render/headless.rs).
//!
//! Drop-in: copy this file to `src/render/cuda_tracer.rs`, declare
//! `mod cuda_tracer;` next to `mod path_tracer;`, and link the library from
//! `build.rs`:
//!
//! ```text
//! println!("cargo:rustc-link-search=native=<repo>/path-tracer_gb300/_build");
//! println!("cargo:rustc-link-lib=dylib=pt");
//! ```
//!
//! The reference's GPU structs (`GpuTriangleGeometry` ... `GpuSkyboxAliasEntry`,
//! world.rs:139-537) are `#[repr(C)]` bytemuck types whose layouts equal the
//! `pt_*` structs, so the world's slices are handed to the library by
//! pointer without conversion.  Only the four upload descriptors below are
//! new; their field order and sizes are those of include/pt.h (checked at
//! compile time by the `const` assertions, and against the header by
//! tests/test_rust_binding.py).  This file is not compiled in this
//! repository (no Rust toolchain on the build machine).

#![allow(dead_code)]

use std::ffi::CStr;
use std::os::raw::c_char;
use std::ptr;

use super::world::{
    GpuBvhNode, GpuCamera, GpuMaterial, GpuSceneAliasEntry, GpuSceneUniforms, GpuSkyboxAliasEntry,
    GpuSkyboxUniforms, GpuTriangleAttribute, GpuTriangleGeometry, SceneUpload, SkyboxUpload, WorldUpdates,
};

// ------------------------------------------------------------ C ABI (pt.h)

pub const PT_OK: i32 = 0;
pub const PT_ERR_INVALID_ARG: i32 = 1;
pub const PT_ERR_OUT_OF_LIMITS: i32 = 2;
pub const PT_ERR_OOM: i32 = 3;
pub const PT_ERR_CUDA: i32 = 4;
pub const PT_ERR_TIMEOUT: i32 = 5;
pub const PT_ERR_STATE: i32 = 6;

pub const PT_ATLAS_SIZE: usize = 8192;
pub const PT_MAX_SAMPLES_PER_TRACE: u32 = 16;
pub const PT_TILE_IMAGE: i32 = 0;
pub const PT_TILE_ACCUMULATION: i32 = 1;

/// pt_scene_upload: SceneUpload (world.rs:87-94) with the atlas layers contiguous.
#[repr(C)]
pub struct PtSceneUpload {
    pub geometries: *const GpuTriangleGeometry,
    pub attributes: *const GpuTriangleAttribute,
    pub triangle_count: u64,
    pub materials: *const GpuMaterial,
    pub material_count: u64,
    pub bvh_nodes: *const GpuBvhNode,
    pub node_count: u64,
    pub srgb_texture_atlases: *const u8,
    pub srgb_atlas_count: u32,
    pub linear_texture_atlases: *const u8,
    pub linear_atlas_count: u32,
}

/// pt_skybox_upload: SkyboxUpload (world.rs:97-101).
#[repr(C)]
pub struct PtSkyboxUpload {
    pub rgba: *const f32,
    pub uniforms: GpuSkyboxUniforms,
    pub alias_table: *const GpuSkyboxAliasEntry,
    pub alias_count: u64,
}

/// pt_material_update: one (index, GpuMaterial) pair of WorldUpdates::materials.
#[repr(C)]
pub struct PtMaterialUpdate {
    pub index: u32,
    pub material: GpuMaterial,
}

/// pt_world_updates: WorldUpdates (world.rs:75-84); a null pointer means "unchanged".
#[repr(C)]
pub struct PtWorldUpdates {
    pub scene: *const PtSceneUpload,
    pub skybox: *const PtSkyboxUpload,
    pub camera: *const GpuCamera,
    pub materials: *const PtMaterialUpdate,
    pub material_update_count: u64,
    pub scene_uniforms: *const GpuSceneUniforms,
    pub scene_alias_table: *const GpuSceneAliasEntry,
    pub scene_alias_count: u64,
    pub skybox_uniforms: *const GpuSkyboxUniforms,
    pub reset_accumulation: i32,
}

/// pt_ctx: opaque context (one CUDA stream, not thread-safe).
#[repr(C)]
pub struct PtCtx {
    _private: [u8; 0],
}

// the layouts of include/pt.h on a 64-bit target (pt_layout_check.cpp asserts the same sizes in C)
const _: () = assert!(std::mem::size_of::<PtSceneUpload>() == 88);
const _: () = assert!(std::mem::size_of::<PtSkyboxUpload>() == 40);
const _: () = assert!(std::mem::size_of::<PtMaterialUpdate>() == 228);
const _: () = assert!(std::mem::size_of::<PtWorldUpdates>() == 80);
const _: () = assert!(std::mem::size_of::<GpuMaterial>() == 224);
const _: () = assert!(std::mem::size_of::<GpuCamera>() == 64);

extern "C" {
    pub fn pt_create(device: i32, updates: *const PtWorldUpdates, tile_width: u32, tile_height: u32,
                     out: *mut *mut PtCtx) -> i32;
    pub fn pt_destroy(ctx: *mut PtCtx);
    pub fn pt_apply_updates(ctx: *mut PtCtx, updates: *const PtWorldUpdates) -> i32;
    pub fn pt_set_tile(ctx: *mut PtCtx, image_size: *const u32, origin: *const u32, size: *const u32) -> i32;
    pub fn pt_set_max_bounces(ctx: *mut PtCtx, max_bounces: u32) -> i32;
    pub fn pt_max_bounces(ctx: *const PtCtx) -> u32;
    pub fn pt_sample_count(ctx: *const PtCtx) -> u32;
    pub fn pt_trace(ctx: *mut PtCtx, sample_count: u32, traced: *mut u32) -> i32;
    pub fn pt_read_tile(ctx: *mut PtCtx, which: i32, host_rgba: *mut f32) -> i32;
    pub fn pt_display_tile(ctx: *mut PtCtx, host_rgba8: *mut u8) -> i32;
    pub fn pt_synchronize(ctx: *mut PtCtx, timeout_ms: u32) -> i32;
    pub fn pt_last_error(ctx: *const PtCtx) -> *const c_char;
    pub fn pt_set_precision(ctx: *mut PtCtx, flags: u32) -> i32;
}

// --------------------------------------------------------- marshalling

/// Host memory that must outlive one pt_create / pt_apply_updates call: the
/// descriptors, the material pairs, and the atlas layers made contiguous
/// (the reference keeps one `Vec<u8>` per layer; a single layer is passed in
/// place, several are copied once into one buffer).
struct Marshalled {
    scene: Option<PtSceneUpload>,
    skybox: Option<PtSkyboxUpload>,
    materials: Vec<PtMaterialUpdate>,
    srgb: Vec<u8>,
    linear: Vec<u8>,
}

fn opt_ptr<T>(v: &Option<T>) -> *const T {
    v.as_ref().map_or(ptr::null(), |x| x as *const T)
}

/// The layers as one contiguous run of RGBA8 8192x8192 images: (pointer, count), copying into
/// `staging` only when there is more than one layer.
fn atlas_layers(layers: &[Vec<u8>], staging: &mut Vec<u8>) -> anyhow::Result<(*const u8, u32)> {
    let layer_bytes = PT_ATLAS_SIZE * PT_ATLAS_SIZE * 4;
    anyhow::ensure!(layers.iter().all(|l| l.len() == layer_bytes), "texture atlas layer is not 8192x8192 RGBA8");
    let count = u32::try_from(layers.len())?;
    match layers {
        [] => Ok((ptr::null(), 0)),
        [only] => Ok((only.as_ptr(), 1)),
        many => {
            staging.reserve_exact(many.len() * layer_bytes);
            for l in many {
                staging.extend_from_slice(l);
            }
            Ok((staging.as_ptr(), count))
        }
    }
}

impl Marshalled {
    fn new(u: &WorldUpdates) -> anyhow::Result<Self> {
        let mut m = Marshalled { scene: None, skybox: None, materials: Vec::new(), srgb: Vec::new(), linear: Vec::new() };
        if let Some(s) = &u.scene {
            let s: &SceneUpload = s;
            let (srgb, srgb_count) = atlas_layers(s.srgb_texture_atlases, &mut m.srgb)?;
            let (linear, linear_count) = atlas_layers(s.linear_texture_atlases, &mut m.linear)?;
            anyhow::ensure!(s.geometries.len() == s.attributes.len(), "geometry and attribute counts differ");
            m.scene = Some(PtSceneUpload {
                geometries: s.geometries.as_ptr(),
                attributes: s.attributes.as_ptr(),
                triangle_count: s.geometries.len() as u64,
                materials: s.materials.as_ptr(),
                material_count: s.materials.len() as u64,
                bvh_nodes: s.bvh_nodes.as_ptr(),
                node_count: s.bvh_nodes.len() as u64,
                srgb_texture_atlases: srgb,
                srgb_atlas_count: srgb_count,
                linear_texture_atlases: linear,
                linear_atlas_count: linear_count,
            });
        }
        if let Some(k) = &u.skybox {
            let k: &SkyboxUpload = k;
            m.skybox = Some(PtSkyboxUpload {
                rgba: k.rgba.as_ptr(),
                uniforms: k.uniforms,
                alias_table: if k.alias_table.is_empty() { ptr::null() } else { k.alias_table.as_ptr() },
                alias_count: k.alias_table.len() as u64,
            });
        }
        m.materials = u
            .materials
            .iter()
            .map(|(index, material)| Ok(PtMaterialUpdate { index: u32::try_from(*index)?, material: *material }))
            .collect::<anyhow::Result<_>>()?;
        Ok(m)
    }

    /// The pt_world_updates of `u`; valid while `self` and `u` live.
    fn view(&self, u: &WorldUpdates) -> PtWorldUpdates {
        let (alias, alias_count) = match u.scene_alias_table {
            Some(t) => (t.as_ptr(), t.len() as u64),
            None => (ptr::null(), 0),
        };
        PtWorldUpdates {
            scene: opt_ptr(&self.scene),
            skybox: opt_ptr(&self.skybox),
            camera: opt_ptr(&u.camera),
            materials: if self.materials.is_empty() { ptr::null() } else { self.materials.as_ptr() },
            material_update_count: self.materials.len() as u64,
            scene_uniforms: opt_ptr(&u.scene_uniforms),
            scene_alias_table: alias,
            scene_alias_count: alias_count,
            skybox_uniforms: opt_ptr(&u.skybox_uniforms),
            reset_accumulation: u.reset_accumulation as i32,
        }
    }
}

// ------------------------------------------------------------ the tracer

/// The GB300 trace pass behind the reference's PathTracer operations.
pub struct CudaTracer {
    ctx: *mut PtCtx,
    tile: [u32; 2],
}

impl CudaTracer {
    fn check(&self, rc: i32) -> anyhow::Result<()> {
        if rc == PT_OK {
            return Ok(());
        }
        let msg = unsafe { CStr::from_ptr(pt_last_error(self.ctx)) }.to_string_lossy().into_owned();
        anyhow::bail!("trace pass error {rc}: {msg}")
    }

    /// PathTracer::new (path_tracer.rs:69-251): `updates` must be a full upload
    /// (World::take_updates after World::new).  The host slices are copied to
    /// the device before the call returns.
    pub fn new(device: i32, updates: &WorldUpdates, tile: [u32; 2]) -> anyhow::Result<Self> {
        let m = Marshalled::new(updates)?;
        let view = m.view(updates);
        let mut ctx: *mut PtCtx = ptr::null_mut();
        let rc = unsafe { pt_create(device, &view, tile[0], tile[1], &mut ctx) };
        // pt_create reports its message on stderr: no context exists to ask
        anyhow::ensure!(rc == PT_OK && !ctx.is_null(), "pt_create failed with status {rc}");
        Ok(CudaTracer { ctx, tile })
    }

    /// PathTracer::apply_updates (path_tracer.rs:272-282).
    pub fn apply_updates(&mut self, updates: &WorldUpdates) -> anyhow::Result<()> {
        let m = Marshalled::new(updates)?;
        let view = m.view(updates);
        let rc = unsafe { pt_apply_updates(self.ctx, &view) };
        self.check(rc)
    }

    /// PathTracer::set_tile (path_tracer.rs:287-313).
    pub fn set_tile(&mut self, image: [u32; 2], origin: [u32; 2], size: [u32; 2]) -> anyhow::Result<()> {
        let rc = unsafe { pt_set_tile(self.ctx, image.as_ptr(), origin.as_ptr(), size.as_ptr()) };
        self.check(rc)?;
        self.tile = size;
        Ok(())
    }

    /// PathTracer::set_max_bounces / max_bounces (path_tracer.rs:259-269).
    pub fn set_max_bounces(&mut self, max_bounces: u32) -> anyhow::Result<()> {
        let rc = unsafe { pt_set_max_bounces(self.ctx, max_bounces) };
        self.check(rc)
    }
    pub fn max_bounces(&self) -> u32 {
        unsafe { pt_max_bounces(self.ctx) }
    }

    /// PathTracer::sample_count (path_tracer.rs:254-256).
    pub fn sample_count(&self) -> u32 {
        unsafe { pt_sample_count(self.ctx) }
    }

    /// PathTracer::trace (path_tracer.rs:316-351) followed by the wait the
    /// headless loop does with device.poll (headless.rs:247-249): traces at
    /// most 16 samples and returns how many.
    pub fn trace(&mut self, samples: u32) -> anyhow::Result<u32> {
        let mut traced = 0u32;
        let rc = unsafe { pt_trace(self.ctx, samples, &mut traced) };
        self.check(rc)?;
        let rc = unsafe { pt_synchronize(self.ctx, 0) };
        self.check(rc)?;
        Ok(traced)
    }

    /// TileReadback::read (headless.rs:330-384): the tonemapped tile as RGBA8
    /// rows of the tile width.
    pub fn read_rgba8(&mut self, out: &mut [u8]) -> anyhow::Result<()> {
        anyhow::ensure!(out.len() == (self.tile[0] * self.tile[1] * 4) as usize, "buffer is not tile-sized");
        let rc = unsafe { pt_display_tile(self.ctx, out.as_mut_ptr()) };
        self.check(rc)
    }

    /// The storage texture (PT_TILE_IMAGE) or the accumulation sums
    /// (PT_TILE_ACCUMULATION) as RGBA32F rows of the tile width.
    pub fn read_tile(&mut self, which: i32, out: &mut [f32]) -> anyhow::Result<()> {
        anyhow::ensure!(out.len() == (self.tile[0] * self.tile[1] * 4) as usize, "buffer is not tile-sized");
        let rc = unsafe { pt_read_tile(self.ctx, which, out.as_mut_ptr()) };
        self.check(rc)
    }

    /// The compressed form (include/pt_precision.h): 8-wide quantised BVH,
    /// FP16 attributes / BF16 skybox and Kahan sums (flags 7), or FP32 (0).
    pub fn set_precision(&mut self, flags: u32) -> anyhow::Result<()> {
        let rc = unsafe { pt_set_precision(self.ctx, flags) };
        self.check(rc)
    }
}

impl Drop for CudaTracer {
    fn drop(&mut self) {
        unsafe { pt_destroy(self.ctx) }
    }
}
