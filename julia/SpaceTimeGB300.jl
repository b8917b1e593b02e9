# SpaceTimeGB300.jl -- Julia bindings of libspacetime_gb300.so (include/spacetime_gb300.h).
#
# Methods of SpaceTime.jl's own GPU entry points, selected by this package's
# context type (no method of SpaceTime's own types is replaced):
#   render(cam, bh, GB300Sky(sky); disc, width, height, samples, relativistic)
#                                       render, src/raytrace.jl:339
#   GB300Context(sky, w, h; disc, volume)
#                                       MetalPreviewContext, src/metal.jl:129
#   render_draft_mtl(ctx::GB300Context, cam, st; width, height, samples, dt, ...)
#                                       src/metal.jl:2040 (Camera), :2244 (ThinLensCamera),
#                                       and through it the Sampling overload, src/look.jl:248
#   render_depth_mtl(ctx::GB300Context, cam, st; nbuckets, ...)
#                                       src/metal.jl:1945
#   set_starfield!(ctx::GB300Context; ...)
#                                       src/metal.jl:257
#   DiscFluidSim(ctx::GB300Context, vol, disc; ...), step_sim!(sim, ctx; dt, jacobi)
#                                       src/disc_sim.jl:45, 287
# Images come back as Matrix{RGBf}(width, height), the reference's layout.
# This file is not exercised in this repository's CI (no Julia toolchain);
# the same ABI is tested through Python ctypes (tests/test_abi.py and the GPU tests).
module SpaceTimeGB300

using SpaceTime
using SpaceTime: AbstractCamera, AbstractSpacetime, Camera, ThinLensCamera, Schwarzschild, Kerr,
                 AccretionDisc, DiscVolume, spin
import SpaceTime: render, render_draft_mtl, render_depth_mtl, set_starfield!, step_sim!, DiscFluidSim
using Colors: RGB
using Random
using StaticArrays

export GB300Context, GB300Sky

const RGBf = RGB{Float32}
const libst = get(ENV, "SPACETIME_GB300_LIB", joinpath(@__DIR__, "..", "spacetime_gb300", "libspacetime_gb300.so"))

const ST_OK = 0
const ST_SEM_RENDER = 0
const ST_SEM_DRAFT = 1
const ST_EMIT_KEPLER = 0
const ST_EMIT_KS_EXACT = 1
const ST_PREC_FP64 = 0
const ST_PREC_FP32_GUARDED = 1
const ST_PREC_FP32 = 2
const ST_PREC_FP32_GUARDED_DF = 3

struct StCamera
    pos::NTuple{3,Float64}; fwd::NTuple{3,Float64}; right::NTuple{3,Float64}; up::NTuple{3,Float64}
    fov_factor::Float64; velocity::NTuple{3,Float64}
    projection::Cint; fisheye_deg::Float64; aperture_world::Float64; focus_dist::Float64
end
struct StSpacetime; M::Float64; a::Float64; end
struct StDisc
    inner::Float64; outer::Float64; falloff::Float64; wb_temperature::Float64
    table_min::Float64; table_max::Float64; table_size::Cint; emitter::Cint
end
struct StVolume
    density::Ptr{Float32}; nr::Cint; nphi::Cint; nz::Cint
    log_s_in::Float32; log_s_out::Float32; z_max::Float32
    emission_scale::Float32; opacity_scale::Float32; march_stride::Cint
end
mutable struct StRenderParams
    width::Cint; height::Cint; samples::Cint; dt::Float64; nmax::Cint
    semantics::Cint; precision::Cint; schedule::Cint
    r_escape::Float64; tspan::Float64
    relativistic::Cint; exit_landing::Cint; pixel_jitter::Cint; seed::UInt64
    r_guard::Float64; crit_band::Float64; crit_r::Float64; renorm_every::Cint
    surrogate::Cint; surrogate_sigma::Float64
    block_x::Cint; block_y::Cint; chunk_steps::Cint; graph::Cint
    order::Cint; tol::Float64
    refine::Cint; refine_var::Float64; refine_graze::Float64; refine_margin::Cint
    StRenderParams() = new()
end
struct StStarfield
    strength::Float64; texture_weight::Float64; height::Cint; fov_factor::Float64
    density::Float64; fill::Float64; flux::Float64; psf_pixels::Float64
    galactic::NTuple{3,Float64}; concentration::Float64; temp_min::Float64; temp_max::Float64
    seed::Cint; wb_temperature::Float64; saturation::Float64; table_size::Cint
end

check(rc, where) = rc == ST_OK ||
    error("$where: " * unsafe_string(ccall((:st_strerror, libst), Cstring, (Cint,), rc)))

st_camera(cam::Camera; fisheye_deg=0.0, aperture_world=0.0, focus_dist=1.0) =
    StCamera(Tuple(cam.pos), Tuple(cam.fwd), Tuple(cam.right), Tuple(cam.up_local), cam.fov_factor,
             Tuple(cam.velocity), fisheye_deg > 0 ? 1 : 0, fisheye_deg, aperture_world, focus_dist)

st_disc(d::AccretionDisc, emitter) =
    StDisc(d.inner_radius, d.outer_radius, d.density_falloff, d.blackbody.wb_temperature,
           d.blackbody.table_min, d.blackbody.table_max, d.blackbody.table_size, emitter)

function sky_buffer(bg)
    W, H = size(bg)
    buf = Array{Float32,3}(undef, 3, W, H)   # the reference's (3, W, H) layout
    for j in 1:H, i in 1:W
        c = bg[i, j]
        buf[1, i, j] = c.r; buf[2, i, j] = c.g; buf[3, i, j] = c.b
    end
    buf
end

"""GB300 counterpart of MetalPreviewContext: sky, blackbody table and gas on the device."""
mutable struct GB300Context
    handle::Ptr{Cvoid}
    width::Int
    height::Int
    dt::Float64
    vol::Union{Nothing,Array{Float32,3}}
end

function GB300Context(background, width::Int, height::Int; dt::Real=0.1, nmax::Int=1000,
                      disc::Union{AccretionDisc,Nothing}=nothing,
                      volume::Union{DiscVolume,Nothing}=nothing, device::Int=0,
                      emitter::Int=ST_EMIT_KS_EXACT)
    sky = sky_buffer(background)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:st_context_create, libst), Cint, (Ptr{Ptr{Cvoid}}, Ptr{Float32}, Cint, Cint, Cint),
                h, sky, size(sky, 2), size(sky, 3), device), "st_context_create")
    ctx = GB300Context(h[], width, height, dt, nothing)
    finalizer(c -> ccall((:st_context_destroy, libst), Cvoid, (Ptr{Cvoid},), c.handle), ctx)
    if disc !== nothing
        d = Ref(st_disc(disc, emitter))
        check(ccall((:st_context_set_disc, libst), Cint, (Ptr{Cvoid}, Ref{StDisc}), ctx.handle, d),
              "st_context_set_disc")
    end
    if volume !== nothing
        dens = volume.density
        nr, nphi, nz = size(dens)
        v = Ref(StVolume(pointer(dens), nr, nphi, nz, volume.log_s_in, volume.log_s_out, volume.z_max,
                         volume.emission_scale, volume.opacity_scale, 2))
        GC.@preserve dens check(ccall((:st_context_set_volume, libst), Cint, (Ptr{Cvoid}, Ref{StVolume}),
                                      ctx.handle, v), "st_context_set_volume")
    end
    ctx
end

function default_params(semantics)
    p = StRenderParams()
    ccall((:st_render_params_default, libst), Cvoid, (Ref{StRenderParams}, Cint), p, semantics)
    p
end

function st_render!(ctx::GB300Context, cam::StCamera, bh, p::StRenderParams)
    out = Array{Float32,3}(undef, 3, p.width, p.height)
    st = Ref(StSpacetime(bh.M, spin(bh)))
    check(ccall((:st_render, libst), Cint,
                (Ptr{Cvoid}, Ref{StCamera}, Ref{StSpacetime}, Ref{StRenderParams}, Ptr{Float32}, Ptr{Cvoid}),
                ctx.handle, Ref(cam), st, p, out, C_NULL), "st_render")
    img = Matrix{RGBf}(undef, p.width, p.height)
    @inbounds for j in 1:p.height, i in 1:p.width
        img[i, j] = RGBf(out[1, i, j], out[2, i, j], out[3, i, j])
    end
    img
end

"""The sky of a `render` call, marking it for the GB300: `render(cam, bh, GB300Sky(sky); ...)`."""
struct GB300Sky{T}
    background::T
end

"""`render(cam, bh, GB300Sky(sky); disc, width, height, samples, jittered, rng, relativistic)`:
SpaceTime's CPU renderer (src/raytrace.jl:339) on the GPU, with its rules (Keplerian disc,
horizon at 2.00001, r_max = max(5|pos|, 100)).  `solver` is accepted and ignored (the GPU
integrates with RK4 in FP64 by default); `dust`, `volume` and `starfield` are not provided."""
function render(cam::Camera, spacetime::Schwarzschild, sky::GB300Sky;
                disc::Union{AccretionDisc,Nothing}=AccretionDisc(), dust=nothing, volume=nothing,
                width::Int=400, height::Int=200, solver=nothing, samples::Int=1, jittered::Bool=true,
                rng::Random.AbstractRNG=Random.default_rng(), progress::Union{Function,Nothing}=nothing,
                relativistic::Bool=false, starfield=nothing, precision::Int=ST_PREC_FP64)
    (dust === nothing && volume === nothing && starfield === nothing) ||
        throw(ArgumentError("the GB300 render path takes the thin disc only"))
    ctx = GB300Context(sky.background, width, height; disc=disc, emitter=ST_EMIT_KEPLER)
    p = default_params(ST_SEM_RENDER)
    p.width = width; p.height = height; p.samples = samples
    p.pixel_jitter = jittered; p.seed = rand(rng, UInt64)
    p.relativistic = relativistic; p.precision = precision
    img = st_render!(ctx, st_camera(cam), spacetime, p)
    progress === nothing || progress(1.0)
    img
end

"""`set_starfield!(ctx; ...)` (src/metal.jl:257-295), same keywords and defaults."""
function set_starfield!(ctx::GB300Context; strength::Real=1.0, texture_weight::Real=0.0,
                              height::Union{Int,Nothing}=nothing, fov_factor::Real=0.55, density::Real=384,
                              fill::Real=0.5, flux::Real=0.011, psf_pixels::Real=0.5,
                              galactic::NTuple{3,Real}=(0.0, 0.0, 1.0), concentration::Real=3.0,
                              temp_min::Real=3000, temp_max::Real=16000, seed::Integer=12345,
                              wb_temperature::Real=10000.0, saturation::Real=1.0)
    sf = Ref(StStarfield(strength, texture_weight, something(height, ctx.height), fov_factor, density, fill,
                         flux, psf_pixels, Float64.(galactic), concentration, temp_min, temp_max, seed,
                         wb_temperature, saturation, 1024))
    check(ccall((:st_context_set_starfield, libst), Cint, (Ptr{Cvoid}, Ref{StStarfield}), ctx.handle, sf),
          "st_context_set_starfield")
end

"""`render_draft_mtl(ctx, cam, st; ...)` on the GPU with the Metal kernel's rules, same
keywords (src/metal.jl:2040-2054) including `refine`; with `camera_at` (a function of the
shutter fraction s in [0, 1) returning a Camera) it renders motion blur, midpoint or
per-pixel shutter, through st_render_motion."""
function render_draft_mtl(ctx::GB300Context, cam::Camera, bh::AbstractSpacetime; width::Int=1920,
                          height::Int=1080, samples::Int=2, dt::Real=0.02,
                          rng::Random.AbstractRNG=Random.default_rng(),
                          progress::Union{Function,Nothing}=nothing, fisheye_deg::Real=0.0,
                          aperture_world::Real=0.0, focus_dist::Real=1.0, relativistic::Bool=false,
                          camera_at::Union{Function,Nothing}=nothing, per_pixel_shutter::Bool=false,
                          refine::Int=1, refine_var::Real=0.35, refine_graze::Real=0.05,
                          refine_margin::Int=8, pixel_jitter::Bool=true, order::Int=4, tol::Real=1e-4,
                          precision::Int=ST_PREC_FP32)
    p = default_params(ST_SEM_DRAFT)
    p.width = width; p.height = height; p.samples = samples; p.dt = dt; p.seed = rand(rng, UInt64)
    p.relativistic = relativistic; p.precision = precision; p.pixel_jitter = pixel_jitter
    p.order = order; p.tol = tol
    p.refine = refine; p.refine_var = refine_var; p.refine_graze = refine_graze; p.refine_margin = refine_margin
    c = st_camera(cam; fisheye_deg, aperture_world, focus_dist)
    if camera_at === nothing
        img = st_render!(ctx, c, bh, p)
        progress === nothing || progress(1.0)
        return img
    end
    n = samples^2
    fracs = per_pixel_shutter ? [m / n for m in 0:n] : [(m + 0.5) / n for m in 0:(n - 1)]
    poses = [st_camera(camera_at(s); fisheye_deg, aperture_world, focus_dist) for s in fracs]
    out = Array{Float32,3}(undef, 3, width, height)
    st = Ref(StSpacetime(bh.M, spin(bh)))
    check(ccall((:st_render_motion, libst), Cint,
                (Ptr{Cvoid}, Ref{StCamera}, Ptr{StCamera}, Cint, Cint, Ref{StSpacetime}, Ref{StRenderParams},
                 Ptr{Float32}, Ptr{Cvoid}, Ptr{Cvoid}),
                ctx.handle, Ref(c), poses, length(poses), per_pixel_shutter, st, p, out, C_NULL, C_NULL),
          "st_render_motion")
    progress === nothing || progress(1.0)
    [RGBf(out[1, i, j], out[2, i, j], out[3, i, j]) for i in 1:width, j in 1:height]
end

"""`render_draft_mtl(ctx, cam::ThinLensCamera, st; ...)` (src/metal.jl:2244-2252): the lens
as a pinhole camera plus its world-space aperture and focus distance."""
function render_draft_mtl(ctx::GB300Context, cam::ThinLensCamera, bh::AbstractSpacetime; kwargs...)
    fov = (cam.sensor_width / 2.0) / cam.focal_length
    pinhole = Camera(cam.pos, cam.pos + cam.fwd, cam.up_local, fov)
    ap = cam.aperture * cam.focus_distance / cam.focal_length
    return render_draft_mtl(ctx, pinhole, bh; kwargs..., aperture_world=ap, focus_dist=cam.focus_distance)
end

"""`render_depth_mtl(ctx, cam, st; width, height, samples, dt, nbuckets, fisheye_deg, relativistic)`
(src/metal.jl:1935-1990): the (3*nbuckets, width, height) Float32 array of emission binned by path
length, the last bucket the sky."""
function render_depth_mtl(ctx::GB300Context, cam::Camera, bh::AbstractSpacetime; width::Int=1920, height::Int=1080,
                            samples::Int=2, dt::Real=0.02, nbuckets::Int=10, fisheye_deg::Real=0.0,
                            relativistic::Bool=false, precision::Int=ST_PREC_FP32)
    nbuckets >= 3 || throw(ArgumentError("nbuckets must be ≥ 3"))
    p = default_params(ST_SEM_DRAFT)
    p.width = width; p.height = height; p.samples = samples; p.dt = dt
    p.relativistic = relativistic; p.precision = precision; p.pixel_jitter = false
    c = st_camera(cam; fisheye_deg)
    out = Array{Float32,3}(undef, 3 * nbuckets, width, height)
    st = Ref(StSpacetime(bh.M, spin(bh)))
    check(ccall((:st_render_depth, libst), Cint,
                (Ptr{Cvoid}, Ref{StCamera}, Ref{StSpacetime}, Ref{StRenderParams}, Cint, Ptr{Float32}, Ptr{Cvoid}),
                ctx.handle, Ref(c), st, p, nbuckets, out, C_NULL), "st_render_depth")
    out
end

struct StFluidParams
    M::Float64; forcing::Float64; drag::Float64; relax::Float64; scale_height::Float64
end

mutable struct GB300FluidSim
    handle::Ptr{Cvoid}
    ctx::GB300Context
end

"""`DiscFluidSim(vol, disc; M, forcing, drag, relax)` (src/disc_sim.jl:38-91) on the context's gas
grid, as `DiscFluidSim(ctx, vol, disc; ...)`; `vol` is the DiscVolume the context was built with."""
function DiscFluidSim(ctx::GB300Context, vol::DiscVolume, disc::AccretionDisc; M::Real=1.0,
                      forcing::Real=6.0, drag::Real=0.15, relax::Real=0.05)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    fp = Ref(StFluidParams(M, forcing, drag, relax, vol.scale_height))
    check(ccall((:st_fluid_create, libst), Cint, (Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ref{StDisc}, Ref{StFluidParams}),
                h, ctx.handle, Ref(st_disc(disc, ST_EMIT_KS_EXACT)), fp), "st_fluid_create")
    sim = GB300FluidSim(h[], ctx)
    finalizer(s -> ccall((:st_fluid_destroy, libst), Cvoid, (Ptr{Cvoid},), s.handle), sim)
    sim
end

"""`step_sim!(sim, ctx; dt, jacobi)` (src/disc_sim.jl:287-320): one step, queued on the context's
stream, written into its gas texture."""
function step_sim!(sim::GB300FluidSim, ctx::GB300Context; dt::Real=0.05, jacobi::Int=8)
    ctx === sim.ctx || throw(ArgumentError("the solver writes into the context it was built on"))
    check(ccall((:st_fluid_step, libst), Cint, (Ptr{Cvoid}, Cdouble, Cint, Cint, Cint, Ptr{Cfloat}),
                sim.handle, dt, jacobi, 1, 1, C_NULL), "st_fluid_step")
    nothing
end

end # module
