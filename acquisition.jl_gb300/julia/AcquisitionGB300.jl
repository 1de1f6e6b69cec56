# AcquisitionGB300.jl — Julia binding of libacqgb300 (the C ABI in include/acqgb300.h).
#
# Mirrors Acquisition.jl's public API for the FM-DBZP path (plan_acquire src/plan.jl:312-324,
# acquire! src/acquire.jl:54-61,788-797, acquire :838-882, AcquisitionResults
# src/Acquisition.jl:81-109, is_detected / get_num_cells :124-142, cfar_threshold
# src/cfar.jl:64-85) on top of `ccall`, plus the ragged-batch, precision and continuous-correlator
# extensions. The correlator's power has a ChainRulesCore `rrule` whose pullback calls the
# adjoint kernel (the code replica is recomputed on the device, not stored).
#
# Requires: GNSSSignals, Unitful, CUDA (device arrays for the correlator), ChainRulesCore.
# This environment has no Julia; the binding follows the header field by field.
module AcquisitionGB300

export plan_acquire, acquire!, acquire, AcquisitionPlan, AcquisitionResults, is_detected, get_num_cells,
       cfar_threshold, OppositeRowNoiseEstimator, GlobalMeanNoiseEstimator, AcquisitionBatch, run!

using GNSSSignals
using Unitful: Hz, ustrip
import ChainRulesCore
using CUDA

const lib = joinpath(@__DIR__, "..", "acqgb300", "libacqgb300.so")

# ---- structs (layouts of include/acqgb300.h) ----
struct PlanDesc
    system::Int32
    sampling_freq_hz::Float64
    min_doppler_coverage_hz::Float64
    num_coherently_integrated_code_periods::Int32
    bit_edge_search_steps::Int32
    num_noncoherent_accumulations::Int32
    noise_estimator::Int32
    use_secondary_code::Int32
    max_secondary_code_rotations::Int32
    device::Int32
end

struct CResult
    prn::Int32
    secondary_code_phase::Int32
    carrier_doppler_hz::Float64
    code_phase::Float64
    cn0_dbhz::Float64
    noise_power::Float32
    peak_to_noise_ratio::Float32
    peak_power::Float32
    num_noncoherent_integrations::Int32
    peak_doppler_bin::Int32
    peak_code_bin::Int32
    sign_pattern::Int32
    bit_edge::Int32
    detected::Int32
    reserved::Int32
end

struct CorrCell
    prn::Int32
    reserved::Int32
    code_phase::Float64
    doppler_hz::Float64
end

struct CorrResult
    power::Float64
    grad::NTuple{2,Float64}
    hess::NTuple{3,Float64}
    z_re::Float64
    z_im::Float64
    iterations::Int32
    status::Int32
end

function check(st)
    st == 0 && return nothing
    buf = Vector{UInt8}(undef, 4096)
    ccall((:acq_last_error, lib), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    msg = unsafe_string(pointer(buf))
    st in (1, 2, 3) ? throw(ArgumentError(msg)) : error("libacqgb300 status $st: $msg")
end

sysid(::GPSL1CA) = Int32(0)
sysid(::GPSL5I) = Int32(1)
sysid(::GalileoE1B) = Int32(2)

dtype(::Type{ComplexF32}) = Int32(0)
dtype(::Type{Complex{Int16}}) = Int32(1)
dtype(::Type{Complex{Int8}}) = Int32(2)
dtype(::Type{ComplexF64}) = Int32(3)

# ---- plan_acquire / acquire! / acquire ----
struct OppositeRowNoiseEstimator end
struct GlobalMeanNoiseEstimator end
estid(::OppositeRowNoiseEstimator) = Int32(0)
estid(::GlobalMeanNoiseEstimator) = Int32(1)

# acq_geometry: the derived fields of AcquisitionPlan (src/plan.jl:81-174)
struct Geometry
    samples_per_code::Int32
    samples_per_code_eff::Int32
    num_blocks::Int32
    block_size::Int32
    fft_size::Int32
    num_coherently_integrated_code_periods::Int32
    num_data_bits::Int32
    bit_edge_search_steps::Int32
    num_noncoherent_accumulations::Int32
    num_doppler_bins::Int32
    num_secondary_rotations::Int32
    bit_period_codes::Int32
    num_prns::Int32
    path::Int32
    doppler_first_hz::Float64
    doppler_step_hz::Float64
    code_length::Float64
    code_freq_hz::Float64
    center_freq_hz::Float64
    cfar_threshold_pfa001::Float64
end

mutable struct AcquisitionPlan
    h::Ptr{Cvoid}
    system::Any
    sampling_freq::Float64
    avail_prns::Vector{Int}
    geometry::Geometry
    doppler_freqs::AbstractRange
    # per plan PRN: the cached power surface that results with store_power_bins alias (allocated on
    # first use, overwritten by the next acquire! that stores power bins: test/plan.jl:329-355)
    result_buffers::Vector{Union{Nothing,Matrix{Float32}}}
end

# plan.num_blocks, plan.samples_per_code, plan.num_secondary_rotations, ... as in the reference
function Base.getproperty(p::AcquisitionPlan, s::Symbol)
    s in fieldnames(AcquisitionPlan) && return getfield(p, s)
    v = getfield(getfield(p, :geometry), s)
    v isa Int32 ? Int(v) : v
end

function plan_acquire(system, sampling_freq, prns; min_doppler_coverage = 7000Hz,
                      num_coherently_integrated_code_periods = 1, bit_edge_search_steps = 1,
                      num_noncoherent_accumulations = 1, noise_estimator = OppositeRowNoiseEstimator(),
                      use_secondary_code = true, max_secondary_code_rotations = 32, fft_flag = nothing,
                      device = 0)
    fs = Float64(ustrip(Hz, sampling_freq))
    d = Ref(PlanDesc(sysid(system), fs, Float64(ustrip(Hz, min_doppler_coverage)),
                     num_coherently_integrated_code_periods, bit_edge_search_steps,
                     num_noncoherent_accumulations, estid(noise_estimator), use_secondary_code,
                     max_secondary_code_rotations, device))
    p = Int32.(collect(prns))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    # codes = C_NULL: the library's generators; pass GNSSSignals codes (n_prns x code length
    # Int8) to use the package's chips bit for bit.
    check(ccall((:acq_plan_create, lib), Cint, (Ref{PlanDesc}, Ptr{Int32}, Int32, Ptr{Int8}, Ref{Ptr{Cvoid}}),
                d, p, length(p), C_NULL, h))
    g = Ref{Geometry}()
    st = ccall((:acq_plan_get_geometry, lib), Cint, (Ptr{Cvoid}, Ref{Geometry}), h[], g)
    st == 0 || (ccall((:acq_plan_destroy, lib), Cint, (Ptr{Cvoid},), h[]); check(st))
    dop = range(g[].doppler_first_hz * Hz; step = g[].doppler_step_hz * Hz, length = Int(g[].num_doppler_bins))
    plan = AcquisitionPlan(h[], system, fs, Int.(p), g[], dop, Union{Nothing,Matrix{Float32}}[nothing for _ in p])
    finalizer(pl -> ccall((:acq_plan_destroy, lib), Cint, (Ptr{Cvoid},), getfield(pl, :h)), plan)
end

struct AcquisitionResults{S,D<:AbstractRange}
    system::S
    prn::Int
    sampling_frequency::typeof(1.0Hz)
    carrier_doppler::typeof(1.0Hz)
    code_phase::Float64
    secondary_code_phase::Union{Int,Nothing}
    CN0::Float64
    noise_power::Float32
    peak_to_noise_ratio::Float32
    num_noncoherent_integrations::Int
    power_bins::Union{Matrix{Float32},Nothing}
    dopplers::D
    num_blocks::Int
    block_size::Int
    num_secondary_rotations::Int
end

function acquire!(plan::AcquisitionPlan, signal::AbstractVector{T}, prns::AbstractVector{<:Integer};
                  interm_freq = 0.0Hz, subsample_interpolation::Bool = false,
                  store_power_bins::Bool = false) where {T}
    p = Int32.(collect(prns))
    res = Vector{CResult}(undef, length(p))
    nd, nc = plan.num_doppler_bins, plan.samples_per_code_eff
    # per PRN row-major [doppler_row][code_col] from the library (ignored unless stored)
    bins = Vector{Float32}(undef, store_power_bins ? length(p) * nd * nc : 0)
    flags = UInt32(subsample_interpolation) | (UInt32(store_power_bins) << 1)
    check(ccall((:acq_acquire, lib), Cint,
                (Ptr{Cvoid}, Ptr{T}, Int32, Int64, Ptr{Int32}, Int32, Float64, UInt32, Ptr{CResult}, Ptr{Float32}),
                plan.h, signal, dtype(T), length(signal), p, length(p), Float64(ustrip(Hz, interm_freq)), flags,
                res, bins))
    map(enumerate(res)) do (i, r)
        pb = nothing
        if store_power_bins
            slot = findfirst(==(Int(r.prn)), plan.avail_prns)
            buf = plan.result_buffers[slot]
            buf === nothing && (buf = plan.result_buffers[slot] = Matrix{Float32}(undef, nd, nc))
            permutedims!(buf, reshape(view(bins, (i - 1) * nd * nc + 1:i * nd * nc), nc, nd), (2, 1))
            pb = buf
        end
        AcquisitionResults(plan.system, Int(r.prn), plan.sampling_freq * Hz, r.carrier_doppler_hz * Hz, r.code_phase,
                           r.secondary_code_phase < 0 ? nothing : Int(r.secondary_code_phase), r.cn0_dbhz,
                           r.noise_power, r.peak_to_noise_ratio, Int(r.num_noncoherent_integrations), pb,
                           plan.doppler_freqs, plan.num_blocks, plan.block_size, plan.num_secondary_rotations)
    end
end

# single-PRN convenience methods (src/acquire.jl:788-797, :872-882)
acquire!(plan::AcquisitionPlan, signal, prn::Integer; kw...) = only(acquire!(plan, signal, [prn]; kw...))

function acquire(system, signal, sampling_freq, prns::AbstractVector{<:Integer}; interm_freq = 0.0Hz,
                 subsample_interpolation::Bool = false, store_power_bins::Bool = false, plan_kw...)
    acquire!(plan_acquire(system, sampling_freq, prns; plan_kw...), signal, prns; interm_freq,
             subsample_interpolation, store_power_bins)
end
acquire(system, signal, sampling_freq, prn::Integer; kw...) = only(acquire(system, signal, sampling_freq, [prn]; kw...))

function cfar_threshold(pfa, num_cells; num_noncoherent_integrations = 1)
    out = Ref{Float64}(0)
    check(ccall((:acq_cfar_threshold, lib), Cint, (Float64, Int64, Int32, Ref{Float64}), pfa, num_cells,
                num_noncoherent_integrations, out))
    out[]
end

# src/Acquisition.jl:124-142 (the rotation expansion counts, issue #70)
get_num_cells(r::AcquisitionResults) = length(r.dopplers) * r.num_blocks * r.block_size * r.num_secondary_rotations

is_detected(r::AcquisitionResults; pfa = 0.01) =
    r.peak_to_noise_ratio > cfar_threshold(pfa, get_num_cells(r); num_noncoherent_integrations = r.num_noncoherent_integrations)

# ---- ragged batches: many recordings and plans, one CUDA-graph launch per run ----
struct BatchItem                # acq_batch_item
    plan::Ptr{Cvoid}
    dtype::Int32
    n_samples::Int64
    prns::Ptr{Int32}
    n_prns::Int32
    interm_freq_hz::Float64
    flags::UInt32
end

mutable struct AcquisitionBatch
    h::Ptr{Cvoid}
    plans::Vector{AcquisitionPlan}   # kept alive: the batch holds their handles
    prns::Vector{Vector{Int32}}
end

"""
    AcquisitionBatch(items) with items = [(plan, signal, prns), ...] (or with a fourth element,
    the intermediate frequency): captures one CUDA graph over every item; `run!(batch, signals)`
    returns one result vector per item. Signals keep their element type and length per item.
"""
function AcquisitionBatch(items)
    plans = [it[1] for it in items]
    prns = [Int32.(collect(it[3])) for it in items]
    c = [BatchItem(it[1].h, dtype(eltype(it[2])), length(it[2]), pointer(prns[i]), length(prns[i]),
                   Float64(ustrip(Hz, length(it) > 3 ? it[4] : 0.0Hz)), UInt32(0)) for (i, it) in enumerate(items)]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve prns check(ccall((:acq_batch_create, lib), Cint, (Ptr{BatchItem}, Int32, Ref{Ptr{Cvoid}}),
                                  c, length(c), h))
    b = AcquisitionBatch(h[], plans, prns)
    finalizer(x -> ccall((:acq_batch_destroy, lib), Cint, (Ptr{Cvoid},), x.h), b)
end

function run!(b::AcquisitionBatch, signals)
    res = Vector{CResult}(undef, sum(length, b.prns))
    ptrs = [Ptr{Cvoid}(pointer(s)) for s in signals]
    GC.@preserve signals check(ccall((:acq_batch_run, lib), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{CResult}),
                                     b.h, ptrs, res))
    out, k = Vector{Vector{AcquisitionResults}}(), 0
    for (plan, p) in zip(b.plans, b.prns)
        push!(out, [AcquisitionResults(plan.system, Int(r.prn), plan.sampling_freq * Hz, r.carrier_doppler_hz * Hz,
                                       r.code_phase, r.secondary_code_phase < 0 ? nothing : Int(r.secondary_code_phase),
                                       r.cn0_dbhz, r.noise_power, r.peak_to_noise_ratio,
                                       Int(r.num_noncoherent_integrations), nothing, plan.doppler_freqs,
                                       plan.num_blocks, plan.block_size, plan.num_secondary_rotations)
                    for r in res[k + 1:k + length(p)]])
        k += length(p)
    end
    out
end

# ---- plan options (ACQ_OPT_* of include/acqgb300.h: launch shapes, kernel form, precision) ----
const OPTIONS = Dict(:form => 0, :rotation_precision => 1, :mma_scale_log2 => 2, :tile_threads => 3,
                     :tile_blocks => 4, :tile_pad => 5, :column_width => 6, :column_ctas_per_sm => 7,
                     :doppler_precision => 8, :tile_rows => 9, :transform_length => 10, :tile_mma => 11,
                     :column_wait_polls => 12, :search_width => 13, :search_split => 14)

"Set a plan option; returns the value in effect (launch shapes change results only within FP32 rounding)."
function set_option!(plan::AcquisitionPlan, opt::Symbol, value::Integer)
    eff = Ref{Int64}(0)
    check(ccall((:acq_plan_set_option, lib), Cint, (Ptr{Cvoid}, Int32, Int64, Ref{Int64}), plan.h, OPTIONS[opt],
                value, eff))
    eff[]
end

function get_option(plan::AcquisitionPlan, opt::Symbol)
    v = Ref{Int64}(0)
    check(ccall((:acq_plan_get_option, lib), Cint, (Ptr{Cvoid}, Int32, Ref{Int64}), plan.h, OPTIONS[opt], v))
    v[]
end

# ---- tensor-core precision option ----
const PRECISIONS = Dict(:fp32 => 0, :fp16 => 1, :bf16 => 2, :fp16_split => 3, :bf16_split => 4)

function set_rotation_precision!(plan::AcquisitionPlan, prec::Symbol)
    eff = Ref{Int64}(0)
    check(ccall((:acq_plan_set_option, lib), Cint, (Ptr{Cvoid}, Int32, Int64, Ref{Int64}), plan.h, 1,
                PRECISIONS[prec], eff))
    only(k for (k, v) in PRECISIONS if v == eff[])
end

# ---- continuous correlator ----
mutable struct Correlator
    h::Ptr{Cvoid}
    system::Any
    sampling_freq::Float64
end

function Correlator(system, sampling_freq, prns)
    p = Int32.(collect(prns))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:acq_corr_create, lib), Cint, (Int32, Float64, Ptr{Int32}, Int32, Ptr{Int8}, Ref{Ptr{Cvoid}}),
                sysid(system), Float64(ustrip(Hz, sampling_freq)), p, length(p), C_NULL, h))
    c = Correlator(h[], system, Float64(ustrip(Hz, sampling_freq)))
    finalizer(x -> ccall((:acq_corr_destroy, lib), Cint, (Ptr{Cvoid},), x.h), c)
end

stream_ptr() = CUDA.stream().handle

function correlator_eval(c::Correlator, x::CuVector{ComplexF32}, cells::CuVector{CorrCell}; hessian = false)
    out = CuVector{CorrResult}(undef, length(cells))
    check(ccall((:acq_corr_eval, lib), Cint,
                (Ptr{Cvoid}, CuPtr{ComplexF32}, Int32, Int64, Float64, CuPtr{CorrCell}, Int32, Int32,
                 CuPtr{CorrResult}, Ptr{Cvoid}),
                c.h, x, 0, length(x), 0.0, cells, length(cells), hessian, out, stream_ptr()))
    out
end

function correlator_vjp(c::Correlator, n, cells::CuVector{CorrCell}, zbar::CuVector{ComplexF32})
    xbar = CuVector{ComplexF32}(undef, n)
    check(ccall((:acq_corr_vjp_samples, lib), Cint,
                (Ptr{Cvoid}, Int64, Float64, CuPtr{CorrCell}, CuPtr{ComplexF32}, Int32, CuPtr{ComplexF32}, Ptr{Cvoid}),
                c.h, n, 0.0, cells, zbar, length(cells), xbar, stream_ptr()))
    xbar
end

"""
    correlator_power(c, x, prns, code_phases, dopplers) -> Vector{Float64}

P = |z|^2 per cell (src/generate_test_signal.jl:45-68's correlation at continuous code phase
and Doppler). Differentiable: see the `rrule` below.
"""
function correlator_power(c::Correlator, x::CuVector{ComplexF32}, prns, tau::AbstractVector, f::AbstractVector)
    cells = CuVector(CorrCell.(Int32.(prns), Int32(0), Float64.(tau), Float64.(f)))
    r = Array(correlator_eval(c, x, cells))
    [q.power for q in r]
end

function ChainRulesCore.rrule(::typeof(correlator_power), c::Correlator, x::CuVector{ComplexF32}, prns, tau, f)
    cells = CuVector(CorrCell.(Int32.(prns), Int32(0), Float64.(tau), Float64.(f)))
    r = Array(correlator_eval(c, x, cells))
    P = [q.power for q in r]
    function pullback(Pbar)
        pb = collect(Float64, ChainRulesCore.unthunk(Pbar))
        # z-bar = 2 P-bar z ; the kernel recomputes the replica for x-bar
        zbar = CuVector(ComplexF32.(2 .* pb .* [complex(q.z_re, q.z_im) for q in r]))
        xbar = correlator_vjp(c, length(x), cells, zbar)
        taubar = pb .* [q.grad[1] for q in r]
        fbar = pb .* [q.grad[2] for q in r]
        (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), xbar, ChainRulesCore.NoTangent(), taubar, fbar)
    end
    P, pullback
end

"""
    refine!(c, x, cells; max_iterations = 20, tol_chips = 1e-4, tol_hz = 1e-3,
            max_step_chips = 0.25, max_step_hz = 0.25 * fs / length(x))

Batched Newton refinement of every cell in place (beside the grid's parabolic interpolation).
"""
function refine!(c::Correlator, x::CuVector{ComplexF32}, cells::CuVector{CorrCell}; max_iterations = 20,
                 tol_chips = 1e-4, tol_hz = 1e-3, max_step_chips = 0.25, max_step_hz = 0.25 * c.sampling_freq / length(x))
    out = CuVector{CorrResult}(undef, length(cells))
    check(ccall((:acq_corr_refine, lib), Cint,
                (Ptr{Cvoid}, CuPtr{ComplexF32}, Int32, Int64, Float64, CuPtr{CorrCell}, Int32, Int32, Float64,
                 Float64, Float64, Float64, CuPtr{CorrResult}, Ptr{Cvoid}),
                c.h, x, 0, length(x), 0.0, cells, length(cells), max_iterations, tol_chips, tol_hz,
                max_step_chips, max_step_hz, out, stream_ptr()))
    out
end

end # module
