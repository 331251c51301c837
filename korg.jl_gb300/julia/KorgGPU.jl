"""
    KorgGPU

Julia binding of libkorg_gb300.so: drop-in GPU replacements for Korg.jl's hot-path functions,
calling the C ABI declared in include/korg_gb300.h through `ccall`.

    using Korg, KorgGPU
    KorgGPU.line_absorption!(α, linelist, λs, temps, nₑ, n_densities, partition_fns, ξ, α_cntm;
                             cutoff_threshold=3e-4, precision=:mixed)

The host-side work that Korg does before each call (n/U(T) per species with Korg's own
splines, the effective vdW perturber density, the continuum interpolants' knots and values)
is done here in Julia exactly as Korg does it; the kernels receive plain arrays.  The library
path comes from `ENV["KORG_GB300_LIB"]` or the in-tree build location.
"""
module KorgGPU

using Korg

const LIB = get(ENV, "KORG_GB300_LIB",
                joinpath(@__DIR__, "..", "libkorg_gb300.so"))

const KORG_FP64 = Cint(0)
const KORG_MIXED = Cint(1)

# C structs of include/korg_gb300.h (field order and types must match)
struct CLines
    n::Int64
    wl::Ptr{Float64}
    log_gf::Ptr{Float64}
    E_lower::Ptr{Float64}
    gamma_rad::Ptr{Float64}
    gamma_stark::Ptr{Float64}
    vdW1::Ptr{Float64}
    vdW2::Ptr{Float64}
    mass::Ptr{Float64}
    is_mol::Ptr{Int32}
    species::Ptr{Int32}
end

struct CLayers
    L::Int32
    S::Int32
    T::Ptr{Float64}
    ne::Ptr{Float64}
    n_eff_vdW::Ptr{Float64}
    xi::Ptr{Float64}
    n_div_U::Ptr{Float64}
end

struct CCntm
    nk::Int64
    knots::Ptr{Float64}
    vals::Ptr{Float64}
end

mutable struct Context
    ptr::Ptr{Cvoid}
end

function Context(device::Integer=0)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:korg_create, LIB), Cint, (Ptr{Ptr{Cvoid}}, Cint), out, device)
    rc == 0 || error("korg_create failed ($rc)")
    ctx = Context(out[])
    finalizer(c -> ccall((:korg_destroy, LIB), Cvoid, (Ptr{Cvoid},), c.ptr), ctx)
    ctx
end

const _ctx = Ref{Union{Nothing,Context}}(nothing)
default_context() = (_ctx[] === nothing && (_ctx[] = Context(0)); _ctx[])

function check(ctx::Context, rc)
    if rc != 0
        msg = unsafe_string(ccall((:korg_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx.ptr))
        rc == 1 && throw(ArgumentError(msg))
        error("korg_gb300 error $rc: $msg")
    end
end

_prec(p::Symbol) = p === :fp64 ? KORG_FP64 : p === :mixed ? KORG_MIXED :
                   throw(ArgumentError("precision must be :fp64 or :mixed"))

# SoA packing of a Vector{Korg.Line} (src/linelist.jl:5-14); species rows follow `species`.
function _pack_lines(linelist, species)
    row = Dict(s => Int32(i - 1) for (i, s) in enumerate(species))
    wl = Float64[l.wl for l in linelist]
    loggf = Float64[l.log_gf for l in linelist]
    El = Float64[l.E_lower for l in linelist]
    grad = Float64[l.gamma_rad for l in linelist]
    gst = Float64[l.gamma_stark for l in linelist]
    v1 = Float64[l.vdW[1] for l in linelist]
    v2 = Float64[l.vdW[2] for l in linelist]
    mass = Float64[Korg.get_mass(l.species) for l in linelist]
    ismol = Int32[Korg.ismolecule(l.species) for l in linelist]
    spec = Int32[row[l.species] for l in linelist]
    (wl, loggf, El, grad, gst, v1, v2, mass, ismol, spec)
end

_clines(a) = CLines(length(a[1]), pointer.(a)...)

# the continuum callables Korg builds in synthesize are Interpolations.jl linear interpolants
# over the continuum grid; a constant function per layer (synthesize.jl:266) maps to nk = 1.
function _pack_cntm(α_cntm, L, wl_probe)
    if all(f -> f isa Function && !hasproperty(f, :itp), α_cntm)
        return [0.0], reshape(Float64[f(wl_probe) for f in α_cntm], 1, L)
    end
    knots = collect(Float64, first(α_cntm).itp.knots[1])
    vals = Matrix{Float64}(undef, length(knots), L)   # column l = layer l (vals[l * nk + k])
    for (l, f) in enumerate(α_cntm)
        vals[:, l] .= f.(knots)
    end
    knots, vals
end

"""
    line_absorption!(α, linelist, λs, temps, nₑ, n_densities, partition_fns, ξ, α_cntm;
                     cutoff_threshold=3e-4, precision=:fp64, ctx=default_context())

GPU drop-in for `Korg.line_absorption!` (src/line_absorption.jl:33-129).
"""
function line_absorption!(α::Matrix{Float64}, linelist, λs::Korg.Wavelengths, temps, nₑ, n_densities,
                          partition_fns, ξ, α_cntm; cutoff_threshold=3e-4, precision=:fp64,
                          ctx=default_context())
    length(linelist) == 0 && return zeros(length(λs))
    L = length(temps)
    species = unique([l.species for l in linelist])
    n_div_U = Matrix{Float64}(undef, L, length(species))   # n_div_U[s * L + l]
    for (i, s) in enumerate(species)
        n_div_U[:, i] .= n_densities[s] ./ partition_fns[s].(log.(temps))
    end
    c_He = (1.38375 / 4.50711)^0.4 * (Korg.atomic_masses[2] / Korg.atomic_masses[1])^-0.3
    c_H2 = (5.503 / 4.50711)^0.4 * 2^-0.3
    n_eff = @. n_densities[Korg.species"H_I"] + c_He * n_densities[Korg.species"He_I"] +
               c_H2 * n_densities[Korg.species"H2"]
    xi = ξ isa Number ? fill(Float64(ξ), L) : collect(Float64, ξ)
    packed = _pack_lines(linelist, species)
    knots, vals = _pack_cntm(α_cntm, L, first(linelist).wl)
    T = collect(Float64, temps)
    ne = collect(Float64, nₑ)
    wls = collect(Float64, λs.all_wls)
    nevals = Ref{Int64}(0)
    GC.@preserve packed n_div_U n_eff xi knots vals T ne wls begin
        lines = Ref(_clines(packed))
        lay = Ref(CLayers(L, length(species), pointer(T), pointer(ne), pointer(n_eff), pointer(xi),
                          pointer(n_div_U)))
        cn = Ref(CCntm(length(knots), pointer(knots), pointer(vals)))
        rc = ccall((:korg_line_absorption, LIB), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int64, Ref{CLines}, Ref{CLayers}, Ref{CCntm},
                    Float64, Cint, Ref{Int64}),
                   ctx.ptr, α, wls, length(wls), lines, lay, cn, cutoff_threshold, _prec(precision), nevals)
        check(ctx, rc)
    end
    nothing
end

"""
    radiative_transfer(atm::Korg.PlanarAtmosphere, α, S, μ_points; α_ref, ctx=default_context())

GPU drop-in for the default planar path of `Korg.RadiativeTransfer.radiative_transfer`
(RadiativeTransfer.jl:62-139): anchored τ and the exponential-integral flux.
"""
function radiative_transfer(atm::Korg.PlanarAtmosphere, α::Matrix{Float64}, S::Matrix{Float64}, μ_points;
                            α_ref, τ_scheme="anchored", I_scheme="linear_flux_only", ctx=default_context())
    (τ_scheme == "anchored" && I_scheme == "linear_flux_only") ||
        throw(ArgumentError("the GPU path implements the default planar scheme"))
    L, nwl = size(α)
    τ_ref = Float64[l.tau_ref for l in atm.layers]
    aref = collect(Float64, α_ref)
    F = Vector{Float64}(undef, nwl)
    rc = ccall((:korg_radiative_transfer, LIB), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
               ctx.ptr, α, S, L, nwl, τ_ref, aref, F)
    check(ctx, rc)
    F, reshape(F ./ 2π, 1, nwl), [1.0], [1.0]
end

# ---------------------------------------------------------------------------- chemical equilibrium
# korg_equilibrium_tables / korg_chem_layers of include/korg_gb300.h
struct CEqTables
    n_knots::Int32
    lnT::Ptr{Float64}
    U_u::Ptr{Float64}
    U_z::Ptr{Float64}
    chi::Ptr{Float64}
    n_mol::Int32
    atoms::Ptr{Int32}
    charge::Ptr{Int32}
    kind::Ptr{Int32}
    off::Ptr{Int64}
    spl_t::Ptr{Float64}
    spl_u::Ptr{Float64}
    spl_z::Ptr{Float64}
    D00::Ptr{Float64}
    lmr::Ptr{Float64}
end

struct CChemLayers
    L::Int32
    T::Ptr{Float64}
    n_tot::Ptr{Float64}
    ne_model::Ptr{Float64}
    abundances::Ptr{Float64}
    atm::Ptr{Int32}
end

const KORG_ECHEM = 7

"""
    set_equilibrium_tables!(ctx; ionization_energies, partition_funcs, log_equilibrium_constants)

Uploads Korg's statmech data (src/read_statmech_quantities.jl) for `chemical_equilibrium`:
atomic partition-function splines, ionisation energies, the Barklem & Collet log K splines and,
for the polyatomics (whose log K Korg builds as closures, :63-90), their atomization energies,
mass ratios and partition-function splines.  Returns the molecules in table order.
"""
function set_equilibrium_tables!(ctx::Context=default_context();
                                 ionization_energies=Korg.ionization_energies,
                                 partition_funcs=Korg.default_partition_funcs,
                                 log_equilibrium_constants=Korg.default_log_equilibrium_constants)
    ref = partition_funcs[Korg.species"H I"]
    nk = length(ref.t)
    U_u, U_z = zeros(nk, 276), zeros(nk, 276)        # column 3(Z-1)+q: row-major [276][nk] in C
    for Z in 1:92, q in 0:2
        (Z == 1 && q == 2) && continue
        spl = partition_funcs[Korg.Species(Korg.Formula(Z), q)]
        U_u[:, 3(Z - 1) + q + 1] .= spl.u
        U_z[:, 3(Z - 1) + q + 1] .= spl.z
    end
    chi = zeros(3, 92)
    for Z in 1:92
        chi[:, Z] .= ionization_energies[Z][1:3]
    end
    D00s = Dict{Korg.Species,Float64}()
    csv = joinpath(pkgdir(Korg), "data", "polyatomic_partition_funcs", "atomization_energies.csv")
    for line in readlines(csv)[2:end]
        name, e = split(line, ",")
        D00s[Korg.Species(name)] = parse(Float64, e) * 0.01036
    end
    mols = collect(keys(log_equilibrium_constants))
    n = length(mols)
    atoms, charge, kind = zeros(Int32, 6, n), zeros(Int32, n), zeros(Int32, n)
    D00, lmr, off = zeros(n), zeros(n), Int64[0]
    t, u, z = Float64[], Float64[], Float64[]
    for (m, mol) in enumerate(mols)
        Zs = Korg.get_atoms(mol.formula)
        atoms[1:length(Zs), m] .= Zs
        charge[m] = mol.charge
        if haskey(D00s, mol)
            kind[m] = 1
            D00[m] = D00s[mol]
            lmr[m] = sum(log10(Korg.atomic_masses[Z]) for Z in Zs) - log10(Korg.get_mass(mol))
            spl = partition_funcs[mol]
        else
            spl = log_equilibrium_constants[mol]
        end
        append!(t, spl.t)
        append!(u, spl.u)
        append!(z, spl.z)
        push!(off, length(t))
    end
    GC.@preserve U_u U_z chi atoms charge kind off t u z D00 lmr begin
        tab = Ref(CEqTables(nk, pointer(collect(Float64, ref.t)), pointer(U_u), pointer(U_z), pointer(chi), n,
                            pointer(atoms), pointer(charge), pointer(kind), pointer(off), pointer(t),
                            pointer(u), pointer(z), pointer(D00), pointer(lmr)))
        check(ctx, ccall((:korg_set_equilibrium_tables, LIB), Cint, (Ptr{Cvoid}, Ref{CEqTables}), ctx.ptr, tab))
    end
    mols
end

"""
    chemical_equilibrium(temps, nₜs, nₑs, absolute_abundances; ctx, molecules)

GPU drop-in for the per-layer `Korg.chemical_equilibrium` loop of `synthesize`
(src/statmech.jl:148-206, src/synthesize.jl:210-219): every layer in one call.  Returns the
electron densities and a Dict species => per-layer number densities, as the loop builds them.
`molecules` is what `set_equilibrium_tables!` returned for this context.
"""
function chemical_equilibrium(temps, nₜs, nₑs, absolute_abundances; molecules, ctx::Context=default_context())
    L = length(temps)
    T, nt, ne = collect(Float64, temps), collect(Float64, nₜs), collect(Float64, nₑs)
    ab = collect(Float64, absolute_abundances)
    dens = Matrix{Float64}(undef, 278 + length(molecules), L)
    status = Vector{Int32}(undef, L)
    rc = GC.@preserve T nt ne ab begin
        lay = Ref(CChemLayers(L, pointer(T), pointer(nt), pointer(ne), pointer(ab), C_NULL))
        ccall((:korg_chemical_equilibrium, LIB), Cint,
              (Ptr{Cvoid}, Ref{CChemLayers}, Int32, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}),
              ctx.ptr, lay, 1, dens, status, C_NULL)
    end
    rc == KORG_ECHEM && throw(Korg.ChemicalEquilibriumError("layer $(findfirst(!=(0), status)): status " *
                                                            "$(status[findfirst(!=(0), status)])"))
    check(ctx, rc)
    nd = Dict{Korg.Species,Vector{Float64}}()
    for Z in 1:92, q in 0:2
        nd[Korg.Species(Korg.Formula(Z), q)] = dens[2 + 3(Z - 1) + q, :]
    end
    nd[Korg.species"H-"] = dens[278, :]
    for (m, mol) in enumerate(molecules)
        nd[mol] = dens[278 + m, :]
    end
    dens[1, :], nd
end

# (nₑ, Dict species => per-layer values) <-> the [278 + n_mol, L] layout of the C ABI's densities
function _pack_densities(ne, nd, molecules, L)
    out = zeros(Float64, 278 + length(molecules), L)
    out[1, :] .= ne
    for Z in 1:92, q in 0:2
        v = get(nd, Korg.Species(Korg.Formula(Z), q), nothing)
        v === nothing || (out[2 + 3(Z - 1) + q, :] .= v)
    end
    v = get(nd, Korg.species"H-", nothing)
    v === nothing || (out[278, :] .= v)
    for (m, mol) in enumerate(molecules)
        v = get(nd, mol, nothing)
        v === nothing || (out[278 + m, :] .= v)
    end
    out
end

"""
    chemical_equilibrium_vjp(temps, nₜs, nₑs, absolute_abundances, (nₑ, nd), (n̄ₑ, n̄d); ctx, molecules)

Reverse mode of [`chemical_equilibrium`](@ref) at its solution `(nₑ, nd)`: given cotangents of
the electron density and of each species' densities (a Dict; absent species count as zero),
returns `(T̄, n̄ₜ, āb)`: per-layer dL/dT, dL/dnₜ, and dL/d(absolute abundance) as a 92 × L
matrix.  This is what ForwardDiff computes through the implicit-function method of
`solve_chemical_equilibrium` (src/statmech.jl:307-355).
"""
function chemical_equilibrium_vjp(temps, nₜs, nₑs, absolute_abundances, solution, cotangents;
                                  molecules, ctx::Context=default_context())
    L = length(temps)
    T, nt, ne = collect(Float64, temps), collect(Float64, nₜs), collect(Float64, nₑs)
    ab = collect(Float64, absolute_abundances)
    dens = _pack_densities(solution[1], solution[2], molecules, L)
    gbar = _pack_densities(cotangents[1], cotangents[2], molecules, L)
    dT, dnt, dab = Vector{Float64}(undef, L), Vector{Float64}(undef, L), Matrix{Float64}(undef, 92, L)
    rc = GC.@preserve T nt ne ab begin
        lay = Ref(CChemLayers(L, pointer(T), pointer(nt), pointer(ne), pointer(ab), C_NULL))
        ccall((:korg_chemical_equilibrium_vjp, LIB), Cint,
              (Ptr{Cvoid}, Ref{CChemLayers}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
               Ptr{Float64}),
              ctx.ptr, lay, 1, dens, gbar, dT, dnt, dab)
    end
    rc == KORG_ECHEM && throw(Korg.ChemicalEquilibriumError("singular system in the reverse mode"))
    check(ctx, rc)
    dT, dnt, dab
end

# ---------------------------------------------------------------------------- differentiable path
# korg_synth_inputs / korg_synth_grads of include/korg_gb300.h
struct CSynthInputs
    layers::CLayers
    tau_ref::Ptr{Float64}
    alpha_ref_cntm::Ptr{Float64}
    nH_I::Ptr{Float64}
    nHe_I::Ptr{Float64}
    UH_I::Ptr{Float64}
    ref_wl::Float64
    cntm::CCntm
    hydrogen_lines::Int32
    use_MHD::Int32
    hydrogen_window::Float64
    cutoff_threshold::Float64
end

struct CSynthGrads
    T::Ptr{Float64}; ne::Ptr{Float64}; n_eff_vdW::Ptr{Float64}; xi::Ptr{Float64}; n_div_U::Ptr{Float64}
    nH_I::Ptr{Float64}; nHe_I::Ptr{Float64}; UH_I::Ptr{Float64}; log_gf::Ptr{Float64}
    cntm_vals::Ptr{Float64}; alpha_ref_cntm::Ptr{Float64}
end

"""
    HotPath(fixed inputs of one synthesize call)

Everything `synthesize` computes on the host before the hot path (src/synthesize.jl:159-262)
that is held fixed while fitting: the wavelengths, both line lists (packed), τ_ref, the
hydrogen-line layer inputs and the continuum knots.  `hotpath_flux(hp, T, nₑ, n_eff, ξ,
n_div_U, log_gf, cntm_vals, α_ref_cntm)` is differentiable through `ChainRulesCore.rrule`.
"""
struct HotPath
    wls::Vector{Float64}
    lines::Tuple
    lines5::Tuple
    tau_ref::Vector{Float64}
    nH_I::Vector{Float64}
    nHe_I::Vector{Float64}
    UH_I::Vector{Float64}
    knots::Vector{Float64}
    ref_wl::Float64
    hydrogen_lines::Bool
    use_MHD::Bool
    hydrogen_window::Float64
    cutoff_threshold::Float64
    precision::Symbol
end

function _with_inputs(f, hp::HotPath, T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref)
    L = length(T)
    lines = (hp.lines[1], collect(Float64, log_gf), hp.lines[3:end]...)
    GC.@preserve hp lines T ne n_eff xi n_div_U cntm_vals aref begin
        lay = CLayers(L, size(n_div_U, 2), pointer(T), pointer(ne), pointer(n_eff), pointer(xi), pointer(n_div_U))
        inp = Ref(CSynthInputs(lay, pointer(hp.tau_ref), pointer(aref), pointer(hp.nH_I), pointer(hp.nHe_I),
                               pointer(hp.UH_I), hp.ref_wl, CCntm(length(hp.knots), pointer(hp.knots),
                                                                  pointer(cntm_vals)),
                               hp.hydrogen_lines, hp.use_MHD, hp.hydrogen_window, hp.cutoff_threshold))
        f(inp, Ref(_clines(lines)), Ref(_clines(hp.lines5)), lines)
    end
end

function hotpath_flux(hp::HotPath, T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref; ctx=default_context())
    nwl = length(hp.wls)
    flux = Vector{Float64}(undef, nwl)
    cntm = Vector{Float64}(undef, nwl)
    _with_inputs(hp, T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref) do inp, l1, l5, _
        rc = ccall((:korg_synthesize, LIB), Cint,
                   (Ptr{Cvoid}, Ref{CSynthInputs}, Ref{CLines}, Ref{CLines}, Ptr{Float64}, Int64, Cint,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                   ctx.ptr, inp, l1, l5, hp.wls, nwl, _prec(hp.precision), flux, cntm, C_NULL, C_NULL)
        check(ctx, rc)
    end
    flux, cntm
end

using ChainRulesCore

function ChainRulesCore.rrule(::typeof(hotpath_flux), hp::HotPath, T, ne, n_eff, xi, n_div_U, log_gf,
                              cntm_vals, aref; ctx=default_context())
    y = hotpath_flux(hp, T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref; ctx=ctx)
    function hotpath_pullback(ȳ)
        dF = collect(Float64, unthunk(ȳ[1]) isa AbstractZero ? zeros(length(hp.wls)) : unthunk(ȳ[1]))
        dC = collect(Float64, unthunk(ȳ[2]) isa AbstractZero ? zeros(length(hp.wls)) : unthunk(ȳ[2]))
        g = map(similar ∘ (x -> collect(Float64, x)), (T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref))
        _with_inputs(hp, T, ne, n_eff, xi, n_div_U, log_gf, cntm_vals, aref) do inp, l1, l5, _
            GC.@preserve g dF dC begin
                grads = Ref(CSynthGrads(pointer(g[1]), pointer(g[2]), pointer(g[3]), pointer(g[4]), pointer(g[5]),
                                        C_NULL, C_NULL, C_NULL, pointer(g[6]), pointer(g[7]), pointer(g[8])))
                rc = ccall((:korg_synthesize_vjp, LIB), Cint,
                           (Ptr{Cvoid}, Ref{CSynthInputs}, Ref{CLines}, Ref{CLines}, Ptr{Float64}, Int64, Cint,
                            Ptr{Float64}, Ptr{Float64}, Ref{CSynthGrads}, Cint),
                           ctx.ptr, inp, l1, l5, hp.wls, length(hp.wls), _prec(hp.precision), dF, dC, grads,
                           Cint(1))
                check(ctx, rc)
            end
        end
        (NoTangent(), NoTangent(), g...)
    end
    y, hotpath_pullback
end

# Cotangent of one per-layer output of chemical_equilibrium as a Float64 vector (zeros if absent).
_cotangent_vector(x, L) = (x = unthunk(x); x isa AbstractZero ? zeros(L) : collect(Float64, x))

"""
ChainRules rule for [`chemical_equilibrium`](@ref): the pullback takes the cotangents of the
electron densities and of the species densities (a Dict species => per-layer values; absent
species count as zero) to the temperatures, the total number densities and the absolute
abundances through `korg_chemical_equilibrium_vjp`, the implicit-function rule the reference's
ForwardDiff method applies (src/statmech.jl:307-355).  The model nₑ is the solver's starting
guess and gets no tangent.
"""
function ChainRulesCore.rrule(::typeof(chemical_equilibrium), temps, nₜs, nₑs, absolute_abundances;
                              molecules, ctx::Context=default_context())
    y = chemical_equilibrium(temps, nₜs, nₑs, absolute_abundances; molecules=molecules, ctx=ctx)
    function chemical_equilibrium_pullback(ȳ)
        ȳ = unthunk(ȳ)
        L = length(temps)
        n̄e = _cotangent_vector(ȳ[1], L)
        n̄d_in = unthunk(ȳ[2])
        n̄d = Dict{Korg.Species,Vector{Float64}}()
        if !(n̄d_in isa AbstractZero)
            for (s, v) in pairs(n̄d_in)
                n̄d[s] = _cotangent_vector(v, L)
            end
        end
        T̄, n̄t, āb = chemical_equilibrium_vjp(temps, nₜs, nₑs, absolute_abundances, y, (n̄e, n̄d);
                                             molecules=molecules, ctx=ctx)
        (NoTangent(), T̄, n̄t, NoTangent(), vec(sum(āb; dims=2)))
    end
    y, chemical_equilibrium_pullback
end

end # module
