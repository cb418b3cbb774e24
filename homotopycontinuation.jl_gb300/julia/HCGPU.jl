# HCGPU.jl — ccall shim that lets HomotopyContinuation.jl hand its total-degree path loop to
# libhcgpu.so (include/hcgpu.h). Drop-in point: the per-path loop of serial_solve /
# threaded_solve (src/solve.jl:603-709) is replaced by one hc_track call per batch; the
# returned records become PathResult values and the reference's own Result(...) does the
# counting (src/result.jl:102-111).
module HCGPU

using HomotopyContinuation
const HC = HomotopyContinuation

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

"""
    gpu_solve(F::System; gamma = cis(2π * rand()), precision = 1)

Total-degree solve of `F` on the GPU; returns the reference's `Result`.
"""
function gpu_solve(F::HC.System; gamma = cis(2π * rand()), precision = 1)
    T = homotopy_tables(F)
    n, npaths = T.n, length(T.starts)
    S = flat_starts(T.starts, n)
    with_handle(precision) do h
        g = ComplexF64(gamma)
        check(ccall((:hc_set_homotopy, libhcgpu), Cint,
                    (Ptr{Cvoid}, Cint, Cint, Ptr{Int32}, Ptr{Int32}, Ptr{Float64}, Cint, Ptr{Int32},
                     Ptr{Int32}, Ptr{Float64}, Float64, Float64),
                    h, n, length(T.Geq), T.Geq, T.Gexp, T.Gcf, length(T.Feq), T.Feq, T.Fexp, T.Fcf,
                    real(g), imag(g)), h)
        res = Vector{HCPathResult}(undef, npaths)
        sol = Vector{Float64}(undef, 2n * npaths)
        check(ccall((:hc_track, libhcgpu), Cint,
                    (Ptr{Cvoid}, Int64, Ptr{Float64}, Cint, Float64, Float64, Float64, Float64,
                     Ptr{HCPathResult}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                    h, npaths, S, 1, 1.0, 0.0, 0.0, 0.0, res, sol, C_NULL, C_NULL), h)
        to_result(res, sol, 0, 0, n, T.starts)
    end
end

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

end # module
