# FFSEngine: Julia-side binding of libffs (the GB300 solver-step engine).
#
# Drop-in for FluidFlowSimulation.jl's time loop: `run_simulation()` reads the same
# `global` file and u1.$start/u2.$start/u3.$start (+ rho.$start) fields, runs
# initialize! and advance_in_time! on the GPU through the C ABI of include/ffs.h, and
# writes Stats.txt, Scales.txt, Numbers.txt, the spectra and the field files in the
# reference formats.
#
# Usage (with libffs.so built):  ENV["FFS_LIB"] = "/path/to/libffs.so"
#   using FFSEngine; run_simulation()
module FFSEngine

using DelimitedFiles

export run_simulation, FFSParams, Engine, initialize!, advance_in_time!, finalize!, getfields

const LIB = get(ENV, "FFS_LIB", joinpath(@__DIR__, "..", "libffs.so"))

# Layout identical to `ffs_params` in include/ffs.h (natural C alignment).
mutable struct FFSParams
    nx::Int32; ny::Int32; nz::Int32
    lx::Float64; ly::Float64; lz::Float64
    nu::Float64; cutoff::Float64
    integrator::Int32; variable_dt::Int32
    cfl::Float64; dt::Float64
    hyperviscosity::Int32; hv_nu::Float64; hv_m::Int32
    les::Int32; smag_c::Float64; filter_width::Float64
    density::Int32; density_pr::Float64; density_gradient::Float64; gravity::Float64
    gravity_dir::Int32
    forcing::Int32; forcing_power::Float64; forcing_kf::Float64
    precision::Int32; dt_stat::Int32; dt_spec::Int32; write_time::Int32
    start::Int64; start_time::Float64
    device::Int32; reference_cfl_slot::Int32
    stats_capacity::Int32; spec_capacity::Int32; kernel_variant::Int32
    autotune::Int32
    les_model::Int32; les_cp::Float64; sandp_cb::Float64
    passive_scalar::Int32; scalar_pr::Float64; scalar_gradient::Float64; scalar_dir::Int32
    plane_forcing::Int32; pf_tf::Float64; pf_alpha::Float64; pf_kf::Float64
    pf_zf_tanh::Int32; pf_qp::Float64; pf_qc::Float64; pf_qkf::Float64
    les_test_width::Float64; les_cmin::Float64; spec_fil::Float64; les_dynp::Int32
    hv_kind::Int32; hv_initk::Float64; hv_endk::Float64; rho_hv::Int32; rho_hv_nu::Float64; rho_hv_m::Int32
    rho_hv_initk::Float64; rho_hv_endk::Float64; rho_les::Int32; rho_les_c::Float64; radix_split::Int32
    FFSParams() = new()
end

function defaults()
    p = FFSParams()
    rc = ccall((:ffs_params_default, LIB), Cint, (Ref{FFSParams},), p)
    rc == 0 || error("ffs_params_default failed")
    return p
end

mutable struct Engine
    h::Ptr{Cvoid}
    p::FFSParams
end

check(e::Engine, rc) = rc == 0 || error(unsafe_string(ccall((:ffs_last_error, LIB), Cstring, (Ptr{Cvoid},), e.h)))

function Engine(p::FFSParams)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:ffs_create, LIB), Cint, (Ref{FFSParams}, Ref{Ptr{Cvoid}}), p, h)
    rc == 0 || error(unsafe_string(ccall((:ffs_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    e = Engine(h[], p)
    finalizer(x -> ccall((:ffs_destroy, LIB), Cvoid, (Ptr{Cvoid},), x.h), e)
    return e
end

readglobal(path = "global") = Dict(Symbol(first(split(l))) => strip(join(split(l)[2:end], " "))
                                   for l in eachline(path) if !isempty(strip(l)) && !startswith(strip(l), "//"))

num(s) = Float64(eval(Meta.parse(s)))

# parameters(d) of src/simulationtypes.jl:242-365 for the keys the engine implements
function parameters(d)
    p = defaults()
    p.nx, p.ny, p.nz = parse(Int32, d[:nx]), parse(Int32, d[:ny]), parse(Int32, d[:nz])
    p.lx, p.ly, p.lz = num(d[:xDomainSize]), num(d[:yDomainSize]), num(d[:zDomainSize])
    p.nu = num(d[:kinematicViscosity])
    haskey(d, :cutoff) && (p.cutoff = num(d[:cutoff]))
    p.start = haskey(d, :start) ? parse(Int, d[:start]) : 0
    p.start_time = haskey(d, :startTime) ? parse(Float64, d[:startTime]) : 0.0
    p.dt_stat = parse(Int32, d[:dtStat]); p.dt_spec = parse(Int32, d[:dtSpec]); p.write_time = parse(Int32, d[:writeTime])
    p.spec_fil = haskey(d, :specFil) ? parse(Float64, d[:specFil]) : 0.0   # Globals.jl:173-178
    p.integrator = Dict("ETD3rdO" => 0, "Adams_Bashforth3rdO" => 1, "Euller" => 2)[get(d, :velocityTimeStep, "ETD3rdO")]
    p.variable_dt = haskey(d, :variableTimestepFlag) ? Int32(parse(Bool, d[:variableTimestepFlag])) : 1
    p.cfl = haskey(d, :cfl) ? parse(Float64, d[:cfl]) : 0.18
    p.dt = haskey(d, :dt) ? num(d[:dt]) : 0.0
    if haskey(d, :hyperViscosity) && d[:hyperViscosity] == "spectralBarrier"   # simulationtypes.jl:294-297
        p.hyperviscosity = 1; p.hv_kind = 1
        p.hv_initk = haskey(d, :initk) ? parse(Float64, d[:initk]) : 0.0
        p.hv_endk = haskey(d, :endk) ? parse(Float64, d[:endk]) : 0.0
    elseif haskey(d, :hyperViscosity)
        p.hyperviscosity = 1; p.hv_nu = parse(Float64, d[:hyperViscosityCoefficient])
        p.hv_m = haskey(d, :hyperViscosityM) ? parse(Int32, d[:hyperViscosityM]) : 2
    end
    if haskey(d, :densityHyperViscosity)   # density_stratification_types.jl:137-148
        if d[:densityHyperViscosity] == "spectralBarrier"
            p.rho_hv = 2
            p.rho_hv_initk = haskey(d, :densityInitk) ? parse(Float64, d[:densityInitk]) : 0.0
            p.rho_hv_endk = haskey(d, :densityEndk) ? parse(Float64, d[:densityEndk]) : 0.0
        else
            p.rho_hv = 1; p.rho_hv_nu = parse(Float64, d[:densityHyperViscosityCoefficient])
            p.rho_hv_m = haskey(d, :densityHyperViscosityM) ? parse(Int32, d[:densityHyperViscosityM]) : 2
        end
    end
    if haskey(d, :lesModel) && (d[:lesModel] in ("dynamicSmagorinsky", "piomelliSmagorinsky", "dynamicSandP",
                                                  "piomelliSandP") ||
                                (d[:lesModel] == "SandP" && get(d, :sLesModel, "") in ("dynamicSmagorinsky",
                                                                                       "piomelliSmagorinsky")))
        m = d[:lesModel]   # les_types.jl:388-455
        p.les_dynp = m == "dynamicSandP" ? 1 : (m == "piomelliSandP" ? 2 : 0)
        p.sandp_cb = m == "SandP" ? (haskey(d, :pConstant) ? num(d[:pConstant]) : 0.09) : 0.0
        base = (p.les_dynp == 0 && m != "SandP") ? m : d[:sLesModel]
        base in ("dynamicSmagorinsky", "piomelliSmagorinsky") || error("lesModel $m needs a dynamic sLesModel")
        p.les = 1; p.les_model = base == "dynamicSmagorinsky" ? 5 : 6
        p.filter_width = haskey(d, :filterWidth) ? num(d[:filterWidth]) : 0.0
        p.les_test_width = haskey(d, :TestFilterWidth) ? num(d[:TestFilterWidth]) : 0.0
        p.les_cmin = haskey(d, :cmin) ? parse(Float64, d[:cmin]) : 0.0
    elseif haskey(d, :lesModel)   # pointwise models of les_types (les_types.jl:360-395)
        m = d[:lesModel]; base = m == "SandP" ? d[:sLesModel] : m
        consts = Dict("Smagorinsky" => (:smagorinskyConstant, 0.17), "Vreman" => (:vremanConstant, 0.032),
                      "productionViscosity" => (:productionConstant, m == "SandP" ? 0.1 : 0.4),
                      "Silvis" => (:silvisConstant, sqrt(0.17)), "stableNonLinear" => (:nlConstant, 0.1))
        haskey(consts, base) || error("lesModel $m is not supported")
        models = Dict("Smagorinsky" => 0, "Vreman" => 1, "productionViscosity" => 2, "Silvis" => 3,
                      "stableNonLinear" => 4)
        key, dflt = consts[base]
        p.les = 1; p.les_model = models[base]
        p.smag_c = haskey(d, key) ? num(d[key]) : dflt
        p.les_cp = haskey(d, :silvisPConstant) ? num(d[:silvisPConstant]) : 5.0
        p.sandp_cb = m == "SandP" ? (haskey(d, :pConstant) ? num(d[:pConstant]) : 0.09) : 0.0
        p.filter_width = haskey(d, :filterWidth) ? num(d[:filterWidth]) :
                         (m == "SandP" && base == "Smagorinsky") ? 2 * (p.lx * 2π / p.nx) / p.cutoff : 0.0
    end
    if haskey(d, :passiveScalar)   # simulationtypes.jl:320-352
        p.passive_scalar = 1; p.scalar_pr = num(d[:scalarPr]); p.scalar_gradient = num(d[:scalarGradient])
        p.scalar_dir = Dict("x" => 0, "y" => 1, "z" => 2)[get(d, :scalarDirection, "z")]
        if haskey(d, :lesModel)    # the scalar's LES diffusion (simulationtypes.jl:334-346)
            vort = get(d, :scalarLesModel, "") == "vorticityDiffusion"
            p.rho_les = vort ? 2 : 1
            p.rho_les_c = vort ? (haskey(d, :scalarVorticityCoefficient) ? parse(Float64, d[:scalarVorticityCoefficient]) : 1.0) : 0.0
        end
    end
    if haskey(d, :densityStratification)
        p.density = 1; p.density_pr = num(d[:Pr]); p.density_gradient = num(d[:densityGradient])
        p.gravity = num(d[:zAcceleration]) / num(d[:referenceDensity])
        p.gravity_dir = Dict("x" => 0, "y" => 1, "z" => 2)[get(d, :gravityDirection, "z")]
        if haskey(d, :densityLesModel)   # density_stratification_types.jl:176-185
            haskey(d, :lesModel) || error("densityLesModel needs lesModel")
            vort = d[:densityLesModel] == "vorticityDiffusion"
            p.rho_les = vort ? 2 : 1
            p.rho_les_c = vort ? (haskey(d, :densityVorticityCoefficient) ? parse(Float64, d[:densityVorticityCoefficient]) : 0.1) : 0.0
        end
    end
    if get(d, :forcing, "") == "isotropicBand"
        p.forcing = 1
        p.forcing_power = haskey(d, :forcingPower) ? num(d[:forcingPower]) : 0.1
        p.forcing_kf = haskey(d, :forcingKf) ? num(d[:forcingKf]) : 2.5
    elseif get(d, :forcing, "") in ("rfForcing", "cRfForcing", "QfForcing", "nRfForcing", "cNRfForcing", "aForcing")
        # forcing_model (forcing_types.jl:335-450)
        p.plane_forcing = Dict("rfForcing" => 1, "cRfForcing" => 2, "QfForcing" => 3, "nRfForcing" => 4,
                               "cNRfForcing" => 5, "aForcing" => 6)[d[:forcing]]
        p.pf_kf = parse(Float64, d[:kf])
        if d[:forcing] == "QfForcing"
            p.pf_qp = parse(Float64, d[:alveliusP]); p.pf_qc = parse(Float64, d[:alveliusC])
            p.pf_qkf = parse(Float64, d[:alveliusKf])
        else
            p.pf_tf = parse(Float64, d[:TF]); p.pf_alpha = parse(Float64, d[:alphac])
            p.pf_zf_tanh = get(d, :Zf, "cutoff") == "cutoff" ? 0 : 1
        end
    end
    p.precision = get(d, :precision, "FP64") == "FP32" ? 1 : 0
    return p
end

readfield(f, nx, ny, nz) = (a = Array{Float64}(undef, nx, ny, nz); read!(f, a); a)

function setfields!(e::Engine, u1, u2, u3, rho = nothing)
    r = rho === nothing ? C_NULL : pointer(rho)
    GC.@preserve u1 u2 u3 rho check(e, ccall((:ffs_set_fields, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint), e.h, u1, u2, u3, r, 0))
end

initialize!(e::Engine) = check(e, ccall((:ffs_initialize, LIB), Cint, (Ptr{Cvoid},), e.h))
advance_in_time!(e::Engine, n::Integer = 1) = check(e, ccall((:ffs_step, LIB), Cint, (Ptr{Cvoid}, Int64), e.h, n))
# the tail of run_simulation (FluidFlowSimulation.jl:46-49): calculate_rhs!, forcing, writestats
finalize!(e::Engine) = check(e, ccall((:ffs_finalize, LIB), Cint, (Ptr{Cvoid},), e.h))
iteration(e::Engine) = ccall((:ffs_iteration, LIB), Int64, (Ptr{Cvoid},), e.h)
forcingshells(e::Engine) = Int(ccall((:ffs_forcing_shells, LIB), Cint, (Ptr{Cvoid},), e.h))
function forcingarray(e::Engine, which::Integer)
    v = zeros(forcingshells(e))
    check(e, ccall((:ffs_forcing_array, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint), e.h, which, v, length(v), 0))
    return v
end
forcingarray!(e::Engine, which::Integer, v::Vector{Float64}) =
    check(e, ccall((:ffs_forcing_array, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint), e.h, which, v, length(v), 1))
simtime(e::Engine) = ccall((:ffs_time, LIB), Float64, (Ptr{Cvoid},), e.h)

function getfields(e::Engine)
    p = e.p
    out = [Array{Float64}(undef, p.nx, p.ny, p.nz) for _ in 1:4]
    rho = (p.density == 1 || p.passive_scalar == 1) ? pointer(out[4]) : C_NULL
    GC.@preserve out check(e, ccall((:ffs_get_fields, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint), e.h, out[1], out[2], out[3], rho, 0))
    return out
end

# pending records: Stats.txt columns, then 9 integral-length plane sums and 4 derivative means
function records(e::Engine)
    nc = ccall((:ffs_record_ncols, LIB), Cint, (Ptr{Cvoid},), e.h)
    n = ccall((:ffs_stats_records, LIB), Int64, (Ptr{Cvoid}, Ptr{Float64}, Int64), e.h, C_NULL, 0)
    buf = Array{Float64}(undef, nc, max(n, 0))
    n > 0 && ccall((:ffs_stats_records, LIB), Int64, (Ptr{Cvoid}, Ptr{Float64}, Int64), e.h, buf, n)
    return buf
end
statsncols(e::Engine) = Int(ccall((:ffs_stats_ncols, LIB), Cint, (Ptr{Cvoid},), e.h))

# the Stats.txt row of the most recent stats iteration (pending records stay pending)
function stats(e::Engine)
    row = Vector{Float64}(undef, statsncols(e))
    check(e, ccall((:ffs_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint), e.h, row, length(row)))
    return row
end

# u spectrum of the current state: (u.specH, u_h.specV + u_v.specV) (spec.jl:316-327, 424-450)
function spectrum(e::Engine)
    lh, lv = Ref{Cint}(0), Ref{Cint}(0)
    check(e, ccall((:ffs_spectrum_lengths, LIB), Cint, (Ptr{Cvoid}, Ref{Cint}, Ref{Cint}), e.h, lh, lv))
    H, V = Vector{Float64}(undef, lh[]), Vector{Float64}(undef, lv[])
    check(e, ccall((:ffs_spectrum, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Int64),
                   e.h, H, V, length(H), length(V)))
    return H, V
end

# Scales.txt / Numbers.txt rows of one record (stats.jl:64-165)
function scalesnumbers(r, names, ns, p::FFSParams)
    col(n) = r[findfirst(==(n), names)]
    u1p2, u2p2, u3p2, k, tdiss = col("u1p2"), col("u2p2"), col("u3p2"), col("k"), col("tdiss")
    s = r[ns+1:ns+9]
    du1dyp2, du1dxp2, du2dyp2, du2dxp2 = r[ns+10], r[ns+11], r[ns+12], r[ns+13]
    Ls = (p.lx, p.ly, p.lz); up2 = (u1p2, u2p2, u3p2)
    L = [Ls[q] * s[3*(c-1)+q] * pi / up2[c] for c in 1:3 for q in 1:3]
    L11, L12, L13, L21, L22, L23, L31, L32, L33 = L
    uh = sqrt((u1p2 + u2p2) / 2); urms = sqrt((u1p2 + u2p2 + u3p2) / 3)
    λ12 = sqrt(2 * u1p2 / du1dyp2); λ21 = sqrt(2 * u2p2 / du2dxp2)
    Lhh = (L11 + L22) / 2; Thh = Lhh / urms
    λl = sqrt(2 * (u1p2 + u2p2) / (du1dxp2 + du2dyp2)); λt = sqrt(2 * (u1p2 + u2p2) / (du1dyp2 + du2dxp2))
    Lhv = (L13 + L23) / 2; Lvv = L33; Lvh = (L31 + L32) / 2
    ν = p.nu
    Lt = sqrt(k * k * k) / tdiss; Tt = k / tdiss; Lk = sqrt(sqrt(ν * ν * ν / tdiss)); Tk = sqrt(ν / tdiss)
    λg = sqrt(15 * ν / tdiss) * urms
    lensv = (Lk, Lt, λg, λl, λt, Lhh, Lvv, Lhv, Lvh, λ12, λ21, L11, L12, L13, L21, L22, L23, L31, L32, L33)
    Reh = uh * Lhh / ν; Reh1 = (Lhh / Lk)^(4 / 3)
    Reλg = urms * λg / ν; Reλg1 = (λg / Lk)^(4 / 3)
    Reλl = urms * λl / ν; Reλl1 = (λl / Lk)^(4 / 3)
    Reλt = urms * λt / ν; Reλt1 = (λt / Lk)^(4 / 3)
    if p.density == 1
        Nb = sqrt((p.gravity_dir == 2 ? p.gravity : 0.0) * p.density_gradient)
        Lb = 2π * urms / Nb; Lo = sqrt(tdiss / (Nb * Nb * Nb)); Lom = sqrt(tdiss / (Nb * Nb * Nb / (8 * pi * pi * pi)))
        Tb = 2π / Nb; Tbm = 1 / Nb
        return (lensv..., Lb, Lo, Lom, Tk, Tt, Thh, Tb, Tbm),
               (Reh, Reh1, Reλg, Reλl, Reλt, Reλg1, Reλl1, Reλt1, (Lo / Lk)^(4 / 3), (Lom / Lk)^(4 / 3),
                2π * uh / (Nb * Lhh), Lhv / Lhh)
    end
    return (lensv..., Tk, Tt, Thh), (Reh, Reh1, Reλl, Reλt, Reλl1, Reλt1)
end

scalesheader(d) = "iteration,time,Lk,Lt,lamg,laml,lamt,Lhh,Lvv,Lhv,Lvh,lam12,lam21,L11,L12,L13,L21,L22,L23,L31,L32,L33" *
                  (d ? ",Lb,Lo,Lom,Tk,Tt,Thh,Tb,Tbm" : ",Tk,Tt,Thh")
numbersheader(d) = "iteration,time,Reh,Reh1,Relamg,Relaml,Relamt,Relamg1,Relaml1,Relamt1" * (d ? ",Reb,Rebm,Frh,Frh1" : "")

# write_spec spectra (spec.jl:1-194): every field as name.specH.i / name.specV.i, plus the
# h + v totals name.specH.i of writespectrum
writepairs(name, k, e) = open(name, "w") do f
    for (a, b) in zip(k, e)
        println(f, a, '\t', b)
    end
end

# tail: the run's final calculate_rhs! writes no forcing spectrum (write_spec_forcing is
# called from advance_in_time!, models.jl:6-9)
function writespectra(e::Engine; tail::Bool = false)
    lenH = Ref{Int32}(0); lenV = Ref{Int32}(0)
    check(e, ccall((:ffs_spectrum_lengths, LIB), Cint, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}), e.h, lenH, lenV))
    nbuf = Vector{UInt8}(undef, 1024)
    nf = ccall((:ffs_spectrum_fields, LIB), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), e.h, nbuf, 1024)
    nf > 0 || error("ffs_spectrum_fields failed")
    names = split(unsafe_string(pointer(nbuf)), ",")
    H, V = Int(lenH[]), Int(lenV[])
    n = ccall((:ffs_spectrum_records, LIB), Int64, (Ptr{Cvoid}, Ptr{Float64}, Int64), e.h, C_NULL, 0)
    n <= 0 && return nothing
    buf = Array{Float64}(undef, 1 + length(names) * (H + V), n)
    ccall((:ffs_spectrum_records, LIB), Int64, (Ptr{Cvoid}, Ptr{Float64}, Int64), e.h, buf, n)
    p = e.p
    KH = p.lx <= p.ly ? collect(0:(p.nx ÷ 2)) ./ p.lx : collect(0:(p.ny ÷ 2)) ./ p.ly
    KRZ = collect(0:(p.nz ÷ 2)) ./ p.lz
    for r in eachcol(buf)
        i = Int(r[1])
        spec(f) = (o = 1 + (f - 1) * (H + V); (r[o+1:o+H], r[o+H+1:o+H+V]))
        for (f, nm) in enumerate(names)
            tail && nm == "forcing_h" && continue
            sH, sV = spec(f)
            writepairs("$nm.specH.$i", KH, sH)
            writepairs("$nm.specV.$i", KRZ, sV)
            if (nm == "buoyancy_v" || nm == "buoyancy_fil_v") && p.gravity_dir == 2 && p.gravity != 0
                rs = nm == "buoyancy_v" ? "rhosource" : "rhosource_fil"   # spec.jl:53-57, 85-95
                writepairs("$rs.specH.$i", KH, sH .* (-p.density_gradient / p.gravity))
                writepairs("$rs.specV.$i", KRZ, sV .* (-p.density_gradient / p.gravity))
            end
        end
        for base in ("u", "vis", "nl", "press", "les", "hvis", "u_fil", "vis_fil", "nl_fil", "press_fil", "hvis_fil")
            ih = findfirst(==("$(base)_h"), names); iv = findfirst(==("$(base)_v"), names)
            (ih === nothing || iv === nothing) && continue
            writepairs("$base.specH.$i", KH, spec(ih)[1] .+ spec(iv)[1])
        end
    end
    return nothing
end

function statsheader(e::Engine)
    buf = Vector{UInt8}(undef, 4096)
    check(e, ccall((:ffs_stats_header, LIB), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int64), e.h, buf, 4096))
    return unsafe_string(pointer(buf))
end

function writeoutput(e::Engine)
    f = getfields(e); i = iteration(e)
    write("u1.$i", f[1]); write("u2.$i", f[2]); write("u3.$i", f[3])
    e.p.density == 1 && write("rho.$i", f[4])
    e.p.passive_scalar == 1 && write("scalar.$i", f[4])   # output.jl: scalar.N
end

# writeoutput's LES fields (output.jl:22-42), captured by the calculate_rhs! of iteration it
const OUTPUT_FIELDS = ("T11", "T12", "T13", "T22", "T23", "cs", "cp", "dflux1", "dflux2", "dflux3")
capture_output!(e::Engine) = check(e, ccall((:ffs_capture_output, LIB), Cint, (Ptr{Cvoid}, Cint), e.h, 1))
function write_les_output(e::Engine, it::Integer)
    p = e.p
    a = Array{Float64}(undef, p.nx, p.ny, p.nz)
    got = Ref{Int64}(-1)
    for (k, name) in enumerate(OUTPUT_FIELDS)
        rc = ccall((:ffs_output_field, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Ref{Int64}), e.h, k - 1, a, got)
        rc == -1 && continue   # not a field of this configuration
        check(e, rc)
        got[] == it || error("LES output capture holds iteration $(got[]), expected $it")
        write("$name.$it", a)
    end
end

# the kz = 0 forcing arrays of writeoutput (output.jl:45-67), by kind
function forcing_state(e::Engine)
    k = e.p.plane_forcing
    if k == 6   # aForcing: R per mode, an (nx/2+1) x ny matrix
        nxh = e.p.nx ÷ 2 + 1
        R = zeros(nxh * e.p.ny)
        check(e, ccall((:ffs_forcing_array, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint), e.h, 5, R, length(R), 0))
        return Dict("R" => reshape(R, nxh, e.p.ny))
    end
    k in (1, 2, 4, 5) || return Dict{String,Any}()
    st = Dict{String,Any}("R" => forcingarray(e, 0), "Eh" => collect(zip(forcingarray(e, 2), forcingarray(e, 4))))
    k in (4, 5) && (st["N"] = forcingarray(e, 3))
    return st
end
write_forcing_output(st, it) = foreach(((name, a),) -> writedlm("$name.$it", a), st)

# run_simulation() of src/FluidFlowSimulation.jl:23-65
function run_simulation()
    d = readglobal()
    p = parameters(d)
    e = Engine(p)
    s = p.start
    u = [open(f -> readfield(f, p.nx, p.ny, p.nz), "u$i.$s") for i in 1:3]
    fname = p.passive_scalar == 1 ? "scalar.$s" : "rho.$s"
    rho = ((p.density == 1 || p.passive_scalar == 1) && isfile(fname)) ?
          open(f -> readfield(f, p.nx, p.ny, p.nz), fname) : nothing
    setfields!(e, u..., rho)
    fil = p.spec_fil != 0   # Stats_fil.txt (stats.jl:14-18, 48-52)
    if s == 0
        open(f -> write(f, statsheader(e), "\n"), "Stats.txt", "w")
        fil && open(f -> write(f, statsheader(e), "\n"), "Stats_fil.txt", "w")
        open(f -> write(f, scalesheader(p.density == 1), "\n"), "Scales.txt", "w")
        open(f -> write(f, numbersheader(p.density == 1), "\n"), "Numbers.txt", "w")
    end
    names = split(statsheader(e), ",")
    ns = statsncols(e)
    initialize!(e)
    if forcingshells(e) > 0   # initialize!(f::RfForcing): targSpectrum.dat, R.$start (forcing_types.jl:66-83)
        if p.plane_forcing != 3 && isfile("targSpectrum.dat")
            data = readdlm("targSpectrum.dat", skipstart = 1)
            kh = forcingarray(e, 2)
            Em = [begin
                      i = searchsortedlast(data[:, 1], k); i = clamp(i, 1, size(data, 1) - 1)
                      t = (k - data[i, 1]) / (data[i + 1, 1] - data[i, 1]); (1 - t) * data[i, 2] + t * data[i + 1, 2]
                  end for k in kh]
            forcingarray!(e, 1, Em)
        end
        isfile("R.$s") && forcingarray!(e, 0, vec(readdlm("R.$s", Float64)))
    end
    if p.plane_forcing == 6 && isfile("R.$s")   # initialize!(f::AForcing) (forcing_types.jl:108-113)
        R = vec(readdlm("R.$s", Float64))
        check(e, ccall((:ffs_forcing_array, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Cint, Cint), e.h, 5, R, length(R), 1))
    end
    p.les == 1 && capture_output!(e)
    total = haskey(d, :nt) ? parse(Int, d[:nt]) : typemax(Int) - s
    lengthtime = haskey(d, :timeDuration) ? parse(Float64, d[:timeDuration]) : Inf   # FluidFlowSimulation.jl:26
    final = s + total
    finaltime = simtime(e) + lengthtime
    function flush(tail = false)
        recs = records(e)
        open("Stats.txt", "a+") do f
            for r in eachcol(recs)
                join(f, (Int(r[1]), r[2:ns]..., "\n"), ",", "")
            end
        end
        fil && open("Stats_fil.txt", "a+") do f   # after the 13 Scales inputs of each record
            for r in eachcol(recs)
                join(f, (Int(r[1]), r[2], r[ns+14:2ns+11]..., "\n"), ",", "")
            end
        end
        for r in eachcol(recs)
            lens, anums = scalesnumbers(r, names, ns, p)
            open(f -> join(f, (Int(r[1]), r[2], lens..., "\n"), ",", ""), "Scales.txt", "a+")
            open(f -> join(f, (Int(r[1]), r[2], anums..., "\n"), ",", ""), "Numbers.txt", "a+")
        end
        writespectra(e; tail = tail)
    end
    # the loop of FluidFlowSimulation.jl:42-44; a time-limited run checks the clock every step
    steps = 0
    pending = -1   # the output iteration whose LES fields the next step captures
    while iteration(e) < final && simtime(e) < finaltime
        it = iteration(e)
        nxt = isfinite(lengthtime) ? it + 1 : min(final, (it ÷ p.write_time + 1) * p.write_time)
        advance_in_time!(e, nxt - it)
        steps += nxt - it
        flush()
        pending >= 0 && (write_les_output(e, pending); pending = -1)
        # the reference writes u.N from calculate_rhs! when the next step starts at N
        if iteration(e) % p.write_time == 0 && iteration(e) < final && simtime(e) < finaltime
            writeoutput(e)
            write_forcing_output(forcing_state(e), iteration(e))
            p.les == 1 && (pending = iteration(e))
        end
    end
    # the tail (FluidFlowSimulation.jl:46-58): a Stats row at the final iteration; the final
    # files come from the tail's calculate_rhs! when the iteration is a multiple of
    # writeTime (before the tail's forcing), else from the explicit writeoutput after it
    in_rhs = iteration(e) % p.write_time == 0 && steps > 0
    pre = in_rhs ? forcing_state(e) : nothing
    finalize!(e)
    flush(true)
    writeoutput(e)
    write_forcing_output(in_rhs ? pre : forcing_state(e), iteration(e))
    p.les == 1 && write_les_output(e, iteration(e))
    if p.plane_forcing == 1   # writedlm("R.$(iteration)", R) (FluidFlowSimulation.jl:60-62)
        writedlm("R.$(iteration(e))", forcingarray(e, 0))
    end
    return e
end

end # module
