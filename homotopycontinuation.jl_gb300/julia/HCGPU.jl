# HCGPU.jl — ccall shim that hands HomotopyContinuation.jl's path tracking to libhcgpu.so
# (include/hcgpu.h).
#
# Drop-in seam: the reference's solver is `Solver{T<:AbstractPathTracker}` (src/solve.jl:41-51)
# and its per-path loop is `solve(S::Solver, starts)` → serial_solve / threaded_solve →
# `track(tracker, S[k]; path_number = k)` (src/solve.jl:547-709). This module defines
#   * `GPUTracker <: AbstractPathTracker` — built from the reference's own `EndgameTracker`
#     (same homotopy, γ, start-system scaling, TrackerOptions and EndgameOptions), with
#     `track(::GPUTracker, x, t₁; path_number)` (src/endgame_tracker.jl:902-914);
#   * `solve(S::Solver{GPUTracker}, starts; ...)` — ONE hc_track call for all starts, then the
#     reference's own `Result(path_results; seed, start_system)` (src/result.jl:102-111);
#   * `GPUPlainTracker` with `track(::GPUPlainTracker, x, t₁, t₀)` → `TrackerResult`
#     (src/tracker.jl:1023-1026);
#   * `solve(args...; kwargs...)` / `solver_startsolutions(args...; kwargs...)` with the
#     reference's signatures, which build the reference's solver (so γ, the seed and the start
#     solutions are the reference's own) and swap its tracker for a GPUTracker.
# Methods are only added for this module's types (no type piracy). `using HCGPU` re-exports
# every exported name of HomotopyContinuation except `solve`, so replacing
# `using HomotopyContinuation` by `using HCGPU` leaves `solve(F; ...)`, `total_degree`,
# `track`, `Tracker` calls and the Result API unchanged.
module HCGPU

using HomotopyContinuation
using Random
const HC = HomotopyContinuation

for name in names(HC)
    name in (:solve, :HomotopyContinuation) && continue
    @eval export $name
end
export solve, solver_startsolutions, GPUTracker, GPUPlainTracker, gpu

const libhcgpu = get(ENV, "HCGPU_LIB", joinpath(@__DIR__, "..", "_build", "libhcgpu.so"))

struct HCOptions  # hc_options
    max_steps::Int32
    extended_precision::Int32
    max_step_size::Float64
    max_initial_step_size::Float64
    min_step_size::Float64
    min_rel_step_size::Float64
    terminate_cond::Float64
    a::Float64
    beta_a::Float64
    beta_omega_p::Float64
    beta_tau::Float64
    strict_beta_tau::Float64
    min_newton_iters::Int32
    max_endgame_steps::Int32
    max_endgame_extended_steps::Int32
    max_winding_number::Int32
    zero_is_at_infinity::Int32
    at_infinity_check::Int32
    only_nonsingular::Int32
    refine_steps::Int32
    endgame_start::Float64
    min_cond::Float64
    min_cond_growth::Float64
    min_coord_growth::Float64
    singular_min_accuracy::Float64
    val_finite_tol::Float64
    val_at_infinity_tol::Float64
    sing_cond::Float64
    sing_accuracy::Float64
    scaling_threshold::Float64
    precision::Int32
    step_control::Int32
    warps_per_cta::Int32
    ctas_per_sm::Int32
    lockstep::Int32   # 1 / 0 / -1 = automatic (hc_options)
    reserved::Int32
end

struct HCPathResult  # hc_path_result
    return_code::Int32
    winding_number::Int32
    t_re::Float64
    t_im::Float64
    accuracy::Float64
    residual::Float64
    cond::Float64
    omega::Float64
    mu::Float64
    tau::Float64
    singular::Int32
    extended_precision::Int32
    extended_precision_used::Int32
    _pad::Int32
    accepted_steps::Int64
    rejected_steps::Int64
    steps_eg::Int64
    path_number::Int64
    last_t::Float64
end

function check(rc, h = C_NULL)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:hc_last_error, libhcgpu), Cstring, (Ptr{Cvoid},), h))
    error("libhcgpu error $rc: $msg")
end

function default_options(; precision = 1)
    o = Ref{HCOptions}()
    check(ccall((:hc_default_options, libhcgpu), Cint, (Ref{HCOptions},), o))
    opt = o[]
    # precision: 0 = FP64, 1 = mixed FP32/FP64
    HCOptions(ntuple(i -> fieldnames(HCOptions)[i] == :precision ? Int32(precision) : getfield(opt, i),
                     fieldcount(HCOptions))...)
end

# term tables (equation, exponent row, coefficient) of a System, 0-based equations
function term_tables(F::HC.System)
    support, coeffs = HC.support_coefficients(F)
    n = length(HC.variables(F))
    eq = Int32[]
    exps = Int32[]
    cf = Float64[]
    for (i, (A, c)) in enumerate(zip(support, coeffs))
        for k in 1:size(A, 2)
            push!(eq, i - 1)
            append!(exps, Int32.(A[:, k]))
            push!(cf, real(ComplexF64(c[k])), imag(ComplexF64(c[k])))
        end
    end
    eq, exps, cf, n
end

# G_i = s_i (x_i^D_i - 1) (src/total_degree.jl:32-117) and the start solutions of F
function homotopy_tables(F::HC.System)
    Feq, Fexp, Fcf, n = term_tables(F)
    support, coeffs = HC.support_coefficients(F)
    D = [maximum(sum(A; dims = 1)) for A in support]
    scaling = [maximum(abs.(float.(c))) for c in coeffs]          # src/total_degree.jl:62
    Geq = Int32[]; Gexp = Int32[]; Gcf = Float64[]
    for i in 1:n
        e = zeros(Int32, n); e[i] = D[i]
        push!(Geq, i - 1, i - 1); append!(Gexp, e, zeros(Int32, n))
        push!(Gcf, scaling[i], 0.0, -scaling[i], 0.0)
    end
    starts = collect(HC.total_degree_start_solutions(D))
    (; n, Geq, Gexp, Gcf, Feq, Fexp, Fcf, starts)
end

function flat_starts(starts, n)
    S = Vector{Float64}(undef, 2n * length(starts))
    for (k, s) in enumerate(starts), i in 1:n
        S[2(n*(k-1)+i)-1] = real(s[i]); S[2(n*(k-1)+i)] = imag(s[i])
    end
    S
end

# records res[r0+1 : r0+npaths], endpoints from element e0 on → the reference's Result
function to_result(res, sol, r0, e0, n, starts)
    codes = instances(HC.EndgameTrackerCode.codes)
    prs = map(1:length(starts)) do k
        r = res[r0+k]
        x = [complex(sol[2(e0+n*(k-1)+i)-1], sol[2(e0+n*(k-1)+i)]) for i in 1:n]
        HC.PathResult(return_code = Symbol(codes[r.return_code+1]), solution = x, t = r.t_re,
                      accuracy = r.accuracy, residual = r.residual, singular = r.singular != 0,
                      condition_jacobian = r.cond,
                      winding_number = r.winding_number == 0 ? nothing : Int(r.winding_number),
                      extended_precision = r.extended_precision != 0, path_number = k,
                      start_solution = starts[k], last_path_point = (x, r.last_t), valuation = nothing,
                      ω = r.omega, μ = r.mu, accepted_steps = r.accepted_steps,
                      rejected_steps = r.rejected_steps, steps_eg = r.steps_eg,
                      extended_precision_used = r.extended_precision_used != 0)
    end
    HC.Result(prs; start_system = :total_degree)
end

function with_handle(f, precision)
    opts = Ref(default_options(precision = precision))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hc_create, libhcgpu), Cint, (Ref{HCOptions}, Ref{Ptr{Cvoid}}), opts, h))
    try
        f(h[])
    finally
        ccall((:hc_destroy, libhcgpu), Cvoid, (Ptr{Cvoid},), h[])
    end
end

# ---------------------------------------------------------------------------------------
# Path trackers for the reference's Solver
# ---------------------------------------------------------------------------------------

# hc_options from the reference's TrackerOptions / TrackerParameters (src/tracker.jl:45-140)
# and EndgameOptions (src/endgame_tracker.jl:47-72), field by field
function hc_options(to::HC.TrackerOptions, eo::Union{Nothing,HC.EndgameOptions}; precision = 1, step_control = 0)
    p = to.parameters
    o = with_fields(default_options(precision = precision);
                    max_steps = to.max_steps, extended_precision = Int(to.extended_precision),
                    max_step_size = to.max_step_size, max_initial_step_size = to.max_initial_step_size,
                    min_step_size = to.min_step_size, min_rel_step_size = to.min_rel_step_size,
                    terminate_cond = to.terminate_cond, a = p.a, beta_a = p.β_a, beta_omega_p = p.β_ω_p,
                    beta_tau = p.β_τ, strict_beta_tau = p.strict_β_τ, min_newton_iters = p.min_newton_iters,
                    step_control = step_control)
    eo === nothing && return o
    with_fields(o; endgame_start = eo.endgame_start, max_endgame_steps = eo.max_endgame_steps,
                max_endgame_extended_steps = eo.max_endgame_extended_steps, min_cond = eo.min_cond,
                min_cond_growth = eo.min_cond_growth, min_coord_growth = eo.min_coord_growth,
                zero_is_at_infinity = Int(eo.zero_is_at_infinity), at_infinity_check = Int(eo.at_infinity_check),
                only_nonsingular = Int(eo.only_nonsingular), singular_min_accuracy = eo.singular_min_accuracy,
                max_winding_number = eo.max_winding_number, val_finite_tol = eo.val_finite_tol,
                val_at_infinity_tol = eo.val_at_infinity_tol, sing_cond = eo.sing_cond,
                sing_accuracy = eo.sing_accuracy, scaling_threshold = eo.scaling_threshold,
                refine_steps = eo.refine_steps)
end

# term tables of any AbstractSystem without free parameters (compiled, interpreted or with fixed
# parameters): System(F) rebuilds its expressions (src/model_kit/abstract_system_homotopy.jl:48)
term_tables(F::HC.AbstractSystem) = term_tables(HC.System(F))

# a handle holding the straight-line homotopy γ t G + (1 - t) F of `H`
# (src/homotopies/straight_line_homotopy.jl:10-68)
function homotopy_handle(H, o::HCOptions)
    H isa HC.StraightLineHomotopy ||
        throw(ArgumentError("libhcgpu tracks straight-line homotopies; got $(typeof(H))"))
    Geq, Gexp, Gcf, n = term_tables(H.start)
    Feq, Fexp, Fcf, nF = term_tables(H.target)
    n == nF && size(H.target, 1) == n || throw(ArgumentError("libhcgpu tracks square systems"))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hc_create, libhcgpu), Cint, (Ref{HCOptions}, Ref{Ptr{Cvoid}}), Ref(o), h))
    check(ccall((:hc_set_homotopy, libhcgpu), Cint,
                (Ptr{Cvoid}, Cint, Cint, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Cint, Ptr{Int32},
                 Ptr{Int32}, Ptr{Float64}, Float64, Float64),
                h[], n, length(Geq), Geq, Gexp, Gcf, length(Feq), Feq, Fexp, Fcf, real(H.γ), imag(H.γ)), h[])
    h[], n
end

struct HCInstruction  # hc_instruction
    in1::Int32
    in2::Int32
    in3::Int32
    in4::Int32
    op::Int32
    output::Int32
end

struct HCSlp  # hc_slp
    n::Int32
    ninstructions::Int32
    instructions::Ptr{HCInstruction}
    nconstants::Int32
    constants::Ptr{Float64}
    variables_offset::Int32
    tape_size::Int32
    outputs::Ptr{Int32}
end

# The reference's own program of F (src/model_kit/instruction_sequence.jl:133-254): its
# instructions, constants and output slots with 0-based tape indices; OpType values are
# hc_op's (include/hcgpu.h). Without `parameters = true`, F must have no parameters (fix them
# first); with it, their slots are returned as `poff`, `np`.
function program_arrays(F::HC.System; parameters::Bool = false)
    seq = HC.ModelKit.instruction_sequence(F)
    parameters || isempty(seq.parameters_range) ||
        throw(ArgumentError("fix the parameters of F before passing its program"))
    isempty(seq.constants_range) || first(seq.constants_range) == 1 ||
        throw(ArgumentError("unexpected tape layout: constants must come first"))
    ins = map(seq.instructions) do I
        a = I.input
        # POW_INT's second input is the exponent itself, kept as is
        fix(k, v) = (I.op == HC.ModelKit.OP_POW_INT && k == 2) ? Int32(v) : Int32(v - 1)
        HCInstruction(fix(1, a[1]), fix(2, a[2]), fix(3, a[3]), fix(4, a[4]), Int32(I.op), Int32(I.output - 1))
    end
    consts = Float64[]
    for c in seq.constants
        z = ComplexF64(c)
        push!(consts, real(z), imag(z))
    end
    n = length(seq.variables_range)
    outputs = zeros(Int32, n)
    for (i, k) in seq.u_assignments
        outputs[i] = Int32(k - 1)
    end
    np = length(seq.parameters_range)
    (; ins, consts, nconst = length(seq.constants), voff = Int32(first(seq.variables_range) - 1),
       tape = Int32(seq.tape_space_needed), outputs, n, np = Int32(np),
       poff = Int32(np > 0 ? first(seq.parameters_range) - 1 : 0))
end

# a handle holding γ t G + (1 - t) F with F the reference's program (hc_set_slp); G is the
# total-degree start system with degrees D and scalings s
function program_handle(F::HC.System, D, s, γ, o::HCOptions)
    A = program_arrays(F)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hc_create, libhcgpu), Cint, (Ref{HCOptions}, Ref{Ptr{Cvoid}}), Ref(o), h))
    GC.@preserve A begin
        P = HCSlp(A.n, length(A.ins), pointer(A.ins), A.nconst, pointer(A.consts), A.voff, A.tape, pointer(A.outputs))
        check(ccall((:hc_set_slp, libhcgpu), Cint,
                    (Ptr{Cvoid}, Ref{HCSlp}, Ptr{Int32}, Ptr{Float64}, Float64, Float64),
                    h[], Ref(P), Int32.(D), Float64.(s), real(γ), imag(γ)), h[])
    end
    h[], A.n
end

# a handle holding the parameter homotopy F(x; t p + (1 - t) q) (hc_set_slp_parameter_homotopy)
# with F the reference's program, parameters and all
function parameter_program_handle(F::HC.System, p, q, o::HCOptions)
    A = program_arrays(F; parameters = true)
    A.np == length(p) == length(q) || throw(ArgumentError("expected $(A.np) start and target parameters"))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hc_create, libhcgpu), Cint, (Ref{HCOptions}, Ref{Ptr{Cvoid}}), Ref(o), h))
    pp = ComplexF64.(p)
    qq = ComplexF64.(q)
    GC.@preserve A pp qq begin
        P = HCSlp(A.n, length(A.ins), pointer(A.ins), A.nconst, pointer(A.consts), A.voff, A.tape, pointer(A.outputs))
        check(ccall((:hc_set_slp_parameter_homotopy, libhcgpu), Cint,
                    (Ptr{Cvoid}, Ref{HCSlp}, Cint, Int32, Ptr{ComplexF64}, Ptr{ComplexF64}),
                    h[], Ref(P), A.np, A.poff, pp, qq), h[])
    end
    h[], A.n
end

"""
    parameters!(T::GPUTracker, p, q)

New start and target parameters for a tracker of a `ParameterHomotopy` (`parameters!`,
src/homotopies/parameter_homotopy.jl:56-62): no recompilation.
"""
function parameters!(T, p, q)
    pp = ComplexF64.(p)
    qq = ComplexF64.(q)
    check(ccall((:hc_set_slp_parameters, libhcgpu), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                T.handle, pp, qq), T.handle)
    T
end

"""
    GPUTracker(eg::EndgameTracker; precision = 1, step_control = 0, program = nothing)

An `AbstractPathTracker` (src/endgame_tracker.jl:8) running the reference's `EndgameTracker`
algorithm for `eg`'s homotopy on the GPU, with `eg`'s γ, start system, `TrackerOptions` and
`EndgameOptions`. `precision`: 0 = complex FP64, 1 = FP32 Jacobians/LU/Taylor with FP64
residuals and decisions. `step_control`: 0 = the reference's rule, 1 = the learned proposal
(load its network with `set_step_model!` first). `program = F` (the `System` `eg` tracks
towards) passes F's own instruction sequence, unexpanded, through `hc_set_slp` instead of its
expanded term table — as the reference evaluates it, which matters where expansion loses
accuracy (e.g. `(x - 10)^6` near its root). A `ParameterHomotopy` (parameters entering F in any
way) always goes through its program (`hc_set_slp_parameter_homotopy`).
"""
mutable struct GPUTracker <: HC.AbstractPathTracker
    handle::Ptr{Cvoid}
    n::Int
    endgame_start::Float64
    function GPUTracker(eg::HC.EndgameTracker; precision = 1, step_control = 0, program = nothing)
        o = hc_options(eg.tracker.options, eg.options; precision = precision, step_control = step_control)
        H = eg.tracker.homotopy
        if H isa HC.ParameterHomotopy
            h, n = parameter_program_handle(HC.ModelKit.System(H.F), H.p, H.q, o)
        elseif program === nothing
            h, n = homotopy_handle(H, o)
        else
            H isa HC.StraightLineHomotopy || throw(ArgumentError("a straight-line homotopy is needed"))
            # G_i = s_i (x_i^D_i - 1): degrees from G's own terms, scalings its parameters
            Geq, Gexp, Gcf, nG = term_tables(H.start)
            D = [maximum(Gexp[(k-1)*nG+i] for k in 1:length(Geq) if Geq[k] == i - 1) for i in 1:nG]
            s = [maximum(abs(Gcf[2k-1]) for k in 1:length(Geq) if Geq[k] == i - 1) for i in 1:nG]
            h, n = program_handle(program, D, s, H.γ, o)
        end
        T = new(h, n, eg.options.endgame_start)
        finalizer(T -> ccall((:hc_destroy, libhcgpu), Cvoid, (Ptr{Cvoid},), T.handle), T)
    end
end

"""
    GPUPlainTracker(tracker::Tracker; precision = 1)

The reference's `Tracker` (src/tracker.jl:452-479) on the GPU: `track(T, x, t₁, t₀)`.
"""
mutable struct GPUPlainTracker
    handle::Ptr{Cvoid}
    n::Int
    function GPUPlainTracker(tr::HC.Tracker; precision = 1)
        o = hc_options(tr.options, nothing; precision = precision)
        h, n = homotopy_handle(tr.homotopy, o)
        T = new(h, n)
        finalizer(T -> ccall((:hc_destroy, libhcgpu), Cvoid, (Ptr{Cvoid},), T.handle), T)
    end
end

"`gpu(eg::EndgameTracker)` / `gpu(tracker::Tracker)`: the GPU tracker of a reference tracker."
gpu(eg::HC.EndgameTracker; kw...) = GPUTracker(eg; kw...)
gpu(tr::HC.Tracker; kw...) = GPUPlainTracker(tr; kw...)

"""
    set_step_model!(T::GPUTracker, params, mean, std; confidence = 0.8, max_factor = 6.0)

Load the step-proposal network (hc_set_step_model): `params` the FP32 parameters
(`hc_mlp_num_params()` values), `mean`/`std` the 12 feature normalisations.
"""
function set_step_model!(T::GPUTracker, params::Vector{Float32}, mean::Vector{Float32}, std::Vector{Float32};
                         confidence = 0.8, max_factor = 6.0)
    check(ccall((:hc_set_step_model, libhcgpu), Cint,
                (Ptr{Cvoid}, Ptr{Float32}, Ptr{Float32}, Ptr{Float32}, Float64, Float64),
                T.handle, params, mean, std, confidence, max_factor), T.handle)
    T
end

# one hc_track call over all start solutions (endgame = 1: EndgameTracker, 0: Tracker)
function track_all(h::Ptr{Cvoid}, n::Int, starts, endgame, t₁, t₀)
    npaths = length(starts)
    S = flat_starts(starts, n)
    res = Vector{HCPathResult}(undef, npaths)
    sol = Vector{Float64}(undef, 2n * npaths)
    val = Vector{Float64}(undef, n * npaths)
    last = Vector{Float64}(undef, 2n * npaths)
    c1, c0 = ComplexF64(t₁), ComplexF64(t₀)
    check(ccall((:hc_track, libhcgpu), Cint,
                (Ptr{Cvoid}, Int64, Ptr{Float64}, Cint, Float64, Float64, Float64, Float64,
                 Ptr{HCPathResult}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                h, npaths, S, endgame, real(c1), imag(c1), real(c0), imag(c0), res, sol, val, last), h)
    res, sol, val, last
end

# PathResult (src/path_result.jl:76-98) of record k, as PathResult(eg) builds it
# (src/endgame_tracker.jl:847-888)
function path_result(r::HCPathResult, sol, val, last, k, n, start, endgame_start, path_number)
    codes = instances(HC.EndgameTrackerCode.codes)
    x = [complex(sol[2(n*(k-1)+i)-1], sol[2(n*(k-1)+i)]) for i in 1:n]
    lp = [complex(last[2(n*(k-1)+i)-1], last[2(n*(k-1)+i)]) for i in 1:n]
    HC.PathResult(return_code = Symbol(codes[r.return_code+1]), solution = x, t = r.t_re,
                  accuracy = r.accuracy, residual = r.residual, singular = r.singular != 0,
                  condition_jacobian = r.cond,
                  winding_number = r.winding_number == 0 ? nothing : Int(r.winding_number),
                  extended_precision = r.extended_precision != 0, path_number = path_number,
                  start_solution = start, last_path_point = (lp, r.last_t),
                  valuation = r.t_re > endgame_start ? nothing : val[n*(k-1)+1:n*k],
                  ω = r.omega, μ = r.mu, accepted_steps = r.accepted_steps,
                  rejected_steps = r.rejected_steps, steps_eg = r.steps_eg,
                  extended_precision_used = r.extended_precision_used != 0)
end

function track_batch(T::GPUTracker, starts, t₁::Real = 1.0)
    res, sol, val, last = track_all(T.handle, T.n, starts, 1, t₁, 0.0)
    [path_result(res[k], sol, val, last, k, T.n, starts[k], T.endgame_start, k) for k in 1:length(starts)]
end

"""
    track(T::GPUTracker, x, t₁ = 1.0; path_number = nothing) -> PathResult

`track(endgame_tracker, x, t₁; path_number)` (src/endgame_tracker.jl:902-914) on the GPU (a
batch of one path; `solve` tracks all paths in one call).
"""
function HC.track(T::GPUTracker, x::AbstractVector, t₁::Real = 1.0; path_number = nothing, kwargs...)
    r = track_batch(T, [x], t₁)[1]
    r.path_number = path_number
    r
end

"""
    track(T::GPUPlainTracker, x, t₁ = 1.0, t₀ = 0.0) -> TrackerResult

`track(tracker, x, t₁, t₀)` (src/tracker.jl:1023-1026) on the GPU.
"""
function HC.track(T::GPUPlainTracker, x::AbstractVector, t₁ = 1.0, t₀ = 0.0; kwargs...)
    res, sol, _, _ = track_all(T.handle, T.n, [x], 0, t₁, t₀)
    r = res[1]
    codes = instances(HC.TrackerCode.codes)
    HC.TrackerResult(Symbol(codes[r.return_code+1]), [complex(sol[2i-1], sol[2i]) for i in 1:T.n],
                     complex(r.t_re, r.t_im), r.accuracy, r.accepted_steps, r.rejected_steps,
                     r.extended_precision != 0, r.extended_precision_used != 0, r.omega, r.mu, r.tau)
end

"""
    solve(S::Solver{GPUTracker}, starts; stop_early_cb, ...) -> Result

The reference's `solve(S::Solver, starts)` (src/solve.jl:547-570) with one GPU call in place
of serial_solve / threaded_solve (src/solve.jl:603-709). With `stop_early_cb`, the results end
after the first successful path (in path order) for which it returns true, as the reference's
serial loop would stop there. `threading` is ignored (the GPU tracks every path at once).
"""
function HC.solve(S::HC.Solver{GPUTracker}, starts::AbstractArray; stop_early_cb = HC.always_false,
                  show_progress::Bool = true, threading::Bool = true, catch_interrupt::Bool = true)
    T = S.trackers[1]
    st = collect(starts)
    prs = track_batch(T, st)
    if stop_early_cb !== HC.always_false
        k = findfirst(r -> HC.is_success(r) && stop_early_cb(r), prs)
        k === nothing || (prs = prs[1:k])
    end
    HC.Result(prs; seed = S.seed, start_system = S.start_system)
end

"""
    solver_startsolutions(args...; precision = 1, step_control = 0, kwargs...)

The reference's `solver_startsolutions` (src/solve.jl:71-214): its `Solver`, γ, seed and start
solutions, with the tracker replaced by a `GPUTracker` when the reference built an
`EndgameTracker` of a straight-line homotopy (total degree, or start/target systems). Other
solvers (polyhedral, parameter or subspace homotopies) are returned unchanged.
"""
function solver_startsolutions(args...; precision = 1, step_control = 0, compile = false, kwargs...)
    solver, starts = HC.solver_startsolutions(args...; compile = compile, kwargs...)
    eg = solver.trackers[1]
    if eg isa HC.EndgameTracker &&
       (eg.tracker.homotopy isa HC.StraightLineHomotopy || eg.tracker.homotopy isa HC.ParameterHomotopy)
        gt = GPUTracker(eg; precision = precision, step_control = step_control)
        return HC.Solver(gt; seed = solver.seed, start_system = solver.start_system), starts
    end
    solver, starts
end

"""
    solve(args...; precision = 1, step_control = 0, kwargs...)

`solve` with the reference's arguments and keywords (src/solve.jl:447-526). Total-degree,
start/target-system and parameter-homotopy solves (`solve(F, starts; start_parameters,
target_parameters)` with one target) track on the GPU (`solver_startsolutions` above); the
polyhedral start system (the reference's default for systems without variable groups) runs
both of its tracking stages on the GPU (`gpu_polyhedral`); many-parameter and subspace solves
go to the reference's own `solve`.
"""
function solve(args...; precision = 1, step_control = 0, seed = rand(UInt32), start_system = nothing,
               target_parameters = nothing, target_subspaces = nothing, start_subspace = nothing,
               show_progress::Bool = true, threading::Bool = true, catch_interrupt::Bool = true,
               stop_early_cb = HC.always_false, kwargs...)
    one_target = target_parameters !== nothing && !isempty(target_parameters) && first(target_parameters) isa Number
    if one_target && target_subspaces === nothing && start_subspace === nothing && length(args) == 2 &&
       args[1] isa HC.System
        solver, starts = solver_startsolutions(args...; precision = precision, step_control = step_control,
                                               seed = seed, target_parameters = target_parameters, kwargs...)
        return HC.solve(solver, collect(starts); stop_early_cb = stop_early_cb, show_progress = show_progress,
                        threading = threading, catch_interrupt = catch_interrupt)
    end
    if target_parameters !== nothing || target_subspaces !== nothing || start_subspace !== nothing ||
       !(length(args) == 1 && args[1] isa HC.System)
        return HC.solve(args...; seed = seed, target_parameters = target_parameters,
                        target_subspaces = target_subspaces, start_subspace = start_subspace,
                        show_progress = show_progress, threading = threading, catch_interrupt = catch_interrupt,
                        stop_early_cb = stop_early_cb,
                        (start_system === nothing ? () : (; start_system = start_system))..., kwargs...)
    end
    F = args[1]
    ss = start_system === nothing ? (isnothing(HC.variable_groups(F)) ? :polyhedral : :total_degree) : start_system
    if ss == :polyhedral
        Random.seed!(seed)
        R = gpu_polyhedral(F; precision = precision)
        return HC.Result(R.path_results; seed = seed, start_system = :polyhedral)
    end
    solver, starts = solver_startsolutions(F; precision = precision, step_control = step_control, seed = seed,
                                           start_system = ss, kwargs...)
    HC.solve(solver, collect(starts); stop_early_cb = stop_early_cb, show_progress = show_progress,
             threading = threading, catch_interrupt = catch_interrupt)
end

"""
    gpu_solve(F::System; gamma = cis(2π * rand()), precision = 1)

Total-degree solve of `F` on the GPU with the given γ; `solve(F; start_system = :total_degree,
gamma)` of this module.
"""
gpu_solve(F::HC.System; gamma = cis(2π * rand()), precision = 1) =
    solve(F; start_system = :total_degree, gamma = gamma, precision = precision)

struct HCInstanceDesc  # hc_instance_desc
    n::Int32
    nG::Int32
    nF::Int32
    reserved::Int32
    G_eq::Ptr{Int32}
    G_exps::Ptr{Int32}
    G_coef::Ptr{Float64}
    F_eq::Ptr{Int32}
    F_exps::Ptr{Int32}
    F_coef::Ptr{Float64}
    gamma_re::Float64
    gamma_im::Float64
    npaths::Int64
end

"""
    gpu_solve_many(Fs::Vector{System}; gammas, precision = 1)

Total-degree solves of many independent systems in one GPU launch (hc_set_batch /
hc_track_batch); returns one `Result` per system, as `map(F -> solve(F), Fs)` would.
"""
function gpu_solve_many(Fs::Vector{<:HC.System}; gammas = [cis(2π * rand()) for _ in Fs], precision = 1)
    Ts = map(homotopy_tables, Fs)
    S = reduce(vcat, [flat_starts(T.starts, T.n) for T in Ts])
    total_paths = sum(length(T.starts) for T in Ts)
    with_handle(precision) do h
        GC.@preserve Ts begin
            descs = [HCInstanceDesc(T.n, length(T.Geq), length(T.Feq), 0, pointer(T.Geq), pointer(T.Gexp),
                                    pointer(T.Gcf), pointer(T.Feq), pointer(T.Fexp), pointer(T.Fcf),
                                    real(ComplexF64(g)), imag(ComplexF64(g)), length(T.starts))
                     for (T, g) in zip(Ts, gammas)]
            tp = Ref{Int64}(0); te = Ref{Int64}(0)
            check(ccall((:hc_set_batch, libhcgpu), Cint,
                        (Ptr{Cvoid}, Cint, Ptr{HCInstanceDesc}, Ptr{Int32}, Ref{Int64}, Ref{Int64}),
                        h, length(descs), descs, C_NULL, tp, te), h)
        end
        res = Vector{HCPathResult}(undef, total_paths)
        sol = Vector{Float64}(undef, length(S))
        check(ccall((:hc_track_batch, libhcgpu), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Cint, Ptr{HCPathResult}, Ptr{Float64}),
                    h, S, 1, res, sol), h)
        r0 = 0; e0 = 0
        map(Ts) do T
            R = to_result(res, sol, r0, e0, T.n, T.starts)
            r0 += length(T.starts); e0 += T.n * length(T.starts)
            R
        end
    end
end

struct HCCertificate  # hc_certificate
    certified::Int32
    realness::Int32
    radius::Float64
    enclosure::Float64
    precision::Int32  # 53, or 106 for the double-word pass
    reserved::Int32
end

"""
    gpu_certify(F::System, solutions)

Krawczyk certificates for approximate solutions of `F` (hc_certify): returns the vector of
`HCCertificate` records (certified, realness 1 = real / 2 = non-real / 0 = undecided, box
radius, enclosure radius), the refined box centres and the enclosure centres.
"""
function gpu_certify(F::HC.System, solutions::AbstractVector{<:AbstractVector})
    T = homotopy_tables(F)
    n, m = T.n, length(solutions)
    S = Vector{Float64}(undef, 2n * m)
    for (k, s) in enumerate(solutions), i in 1:n
        S[2(n*(k-1)+i)-1] = real(s[i]); S[2(n*(k-1)+i)] = imag(s[i])
    end
    realcoef = all(c -> imag(c) == 0, T.Fcf[2:2:end]) ? 1 : 0
    with_handle(0) do h
        check(ccall((:hc_set_homotopy, libhcgpu), Cint,
                    (Ptr{Cvoid}, Cint, Cint, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Cint, Ptr{Int32},
                     Ptr{Int32}, Ptr{Float64}, Float64, Float64),
                    h, n, length(T.Geq), T.Geq, T.Gexp, T.Gcf, length(T.Feq), T.Feq, T.Fexp, T.Fcf,
                    1.0, 0.0), h)
        certs = Vector{HCCertificate}(undef, m)
        centers = Vector{Float64}(undef, 2n * m)
        encl = Vector{Float64}(undef, 2n * m)
        check(ccall((:hc_certify, libhcgpu), Cint,
                    (Ptr{Cvoid}, Int64, Ptr{Float64}, Cint, Ptr{HCCertificate}, Ptr{Float64}, Ptr{Float64}),
                    h, m, S, realcoef, certs, centers, encl), h)
        (certs, centers, encl)
    end
end

# options with some fields replaced (immutable struct: rebuilt field by field)
function with_fields(o::HCOptions; kw...)
    HCOptions(ntuple(i -> convert(fieldtype(HCOptions, i), get(kw, fieldnames(HCOptions)[i], getfield(o, i))),
                     fieldcount(HCOptions))...)
end

"""
    gpu_polyhedral(F::System; only_non_zero = false, precision = 0)

`solve(F; start_system = :polyhedral)` with both tracking stages on the GPU. The mixed cells,
the lifting, the start coefficients and the start solutions are the reference's own
(`polyhedral`, src/polyhedral.jl:197-408, which calls MixedSubdivisions.jl); the toric stage
of `track(::PolyhedralTracker, …)` (src/polyhedral.jl:412-484) becomes two `hc_track_toric`
calls over all paths (the second for the cells whose largest weight is ≥ 10, restarted with
weights rescaled to a maximum of 10), and the coefficient homotopy one `hc_track`.
"""
function gpu_polyhedral(F::HC.System; only_non_zero = false, precision = 0)
    PT, starts = HC.polyhedral(F; only_non_zero = only_non_zero)
    H = PT.toric_tracker.homotopy
    support, lifting = PT.support, PT.lifting
    n = length(support)
    # term tables in the order of the flattened supports (the order of H.weights)
    eq = Int32[]; exps = Int32[]
    for (i, A) in enumerate(support), k in 1:size(A, 2)
        push!(eq, i - 1); append!(exps, Int32.(A[:, k]))
    end
    cfs(c) = reduce(vcat, [[real(z), imag(z)] for z in c])
    ucf = cfs(H.system_coeffs)
    pairs = collect(starts)                     # (cell, x) in the iterator's order
    cells = unique(first.(pairs))
    row = Dict(c => i - 1 for (i, c) in enumerate(cells))
    nT = length(eq)
    W1 = Float64[]; W2 = Float64[]; smax = Float64[]; smin2 = Float64[]
    for c in cells
        _, s_max = HC.update_weights!(H, support, lifting, c; min_weight = 1.0)
        append!(W1, H.weights); push!(smax, s_max)
        s_min, _ = HC.update_weights!(H, support, lifting, c; max_weight = 10.0)
        append!(W2, H.weights); push!(smin2, s_min)
    end
    m = length(pairs)
    rows = Int32[row[p[1]] for p in pairs]
    S = flat_starts(last.(pairs), n)
    tend = [smax[r+1] < 10 ? 1.0 : clamp(0.1^(10 / smax[r+1]), 0.9, 1 - 1e-6) for r in rows]
    res = Vector{HCPathResult}(undef, m)
    sol = Vector{Float64}(undef, 2n * m)
    o = default_options(precision = 0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:hc_create, libhcgpu), Cint, (Ref{HCOptions}, Ref{Ptr{Cvoid}}),
                Ref(with_fields(o; max_initial_step_size = 0.2)), h))
    try
        settoric(W) = check(ccall((:hc_set_toric, libhcgpu), Cint,
                                  (Ptr{Cvoid}, Cint, Cint, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Cint, Ptr{Float64}),
                                  h[], n, nT, eq, exps, ucf, length(cells), W), h[])
        track(k, X, t1, t0, ω, μ, R, Xo) = check(ccall((:hc_track_toric, libhcgpu), Cint,
            (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
             Ptr{Float64}, Ptr{HCPathResult}, Ptr{Float64}),
            h[], k, X, rows[idx_cur[]], t1, t0, ω, μ, R, Xo), h[])
        idx_cur = Ref(collect(1:m))
        settoric(W1)
        track(m, S, zeros(m), tend, fill(20.0, m), fill(1e-12, m), res, sol)
        # restart (src/polyhedral.jl:455-484): TrackerCode success == 1
        idx = [k for k in 1:m if tend[k] < 1 && res[k].return_code == 1]
        if !isempty(idx)
            check(ccall((:hc_set_options, libhcgpu), Cint, (Ptr{Cvoid}, Ref{HCOptions}), h[],
                        Ref(with_fields(o; min_step_size = 0.0))), h[])
            settoric(W2)
            idx_cur[] = idx
            X = reduce(vcat, [sol[2n*(k-1)+1:2n*k] for k in idx])
            tr = [tend[k]^(1 / smin2[rows[k]+1]) for k in idx]
            R2 = Vector{HCPathResult}(undef, length(idx)); X2 = similar(X)
            track(length(idx), X, tr, ones(length(idx)), [res[k].omega for k in idx], [res[k].mu for k in idx],
                  R2, X2)
            for (j, k) in enumerate(idx)
                res[k] = R2[j]; sol[2n*(k-1)+1:2n*k] = X2[2n*(j-1)+1:2n*j]
            end
        end
        # coefficient homotopy t·F(x; start) + (1 − t)·F(x; target) with the endgame
        tcf = cfs(reduce(vcat, PT.generic_tracker.tracker.homotopy.target_coeffs))
        ok = [k for k in 1:m if res[k].return_code == 1]
        check(ccall((:hc_set_options, libhcgpu), Cint, (Ptr{Cvoid}, Ref{HCOptions}), h[],
                    Ref(with_fields(o; precision = precision))), h[])
        check(ccall((:hc_set_homotopy, libhcgpu), Cint,
                    (Ptr{Cvoid}, Cint, Cint, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Cint, Ptr{Int32},
                     Ptr{Int32}, Ptr{Float64}, Float64, Float64),
                    h[], n, nT, eq, exps, ucf, nT, eq, exps, tcf, 1.0, 0.0), h[])
        X = reduce(vcat, [sol[2n*(k-1)+1:2n*k] for k in ok]; init = Float64[])
        R3 = Vector{HCPathResult}(undef, length(ok)); X3 = similar(X)
        check(ccall((:hc_track, libhcgpu), Cint,
                    (Ptr{Cvoid}, Int64, Ptr{Float64}, Cint, Float64, Float64, Float64, Float64,
                     Ptr{HCPathResult}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                    h[], length(ok), X, 1, 1.0, 0.0, 0.0, 0.0, R3, X3, C_NULL, C_NULL), h[])
        to_result(R3, X3, 0, 0, n, [last(pairs[k]) for k in ok])
    finally
        ccall((:hc_destroy, libhcgpu), Cvoid, (Ptr{Cvoid},), h[])
    end
end

end # module
