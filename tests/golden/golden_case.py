"""The reference's standalone OMEXDIA+P example as a one-column ColumnSet,
built through the driver mirror the way examples/standalone/omexdia_p/
main.F90 builds it: init_grid with the run's layers and dzmin, initialize
with sed_nml, init_concentrations with the model's initial values, the
pelagic boundary values and detritus fluxes of run_nml."""
import numpy as np

from sedgpu import driver



def column_set(fx: dict):
    run, sedn, p, cnp = fx["run_nml"], fx["sed_nml"], fx["hzg_omexdia_p"], fx["hzg_omexdia_cnp"]
    K = int(run["numlayers"])
    sed = driver.TypeSed(1, 1, K)
    driver.init_grid(sed.grid, run["dzmin"])
    driver.initialize(sed, dict(diffusivity=sedn["diffusivity"], bioturbation=sedn["bioturbation"],
                                bioturbation_profile=int(sedn["bioturbation_profile"]),
                                bioturbation_depth=sedn["bioturbation_depth"],
                                bioturbation_min=sedn["bioturbation_min"],
                                porosity_max=sedn["porosity_max"],
                                porosity_fac=sedn["porosity_fac"], k_par=sedn["k_par"]))
    sed.dt_min = run["dt_min"]
    sed.bcup_dissolved_variables = int(run["bcup_dissolved_variables"])
    for name in ("rLabile", "rSemilabile", "NCrLdet", "NCrSdet", "PAds", "PAdsODU", "NH3Ads",
                 "CprodMax", "rnit", "ksO2nitri", "rODUox", "ksO2oduox", "ksO2oxic",
                 "ksNO3denit", "kinO2denit", "kinNO3anox", "kinO2anox"):
        sed.bgc[name] = p[name]
    # model order: fdetC sdetC fdetN sdetN fdetP adsP O2 NO3 NH4 ODU PO4; the
    # N detritus values are the cnp block's, adsorbed P starts at po4_init
    init = [p["ldetC_init"], p["sdetC_init"], cnp["ldetN_init"], cnp["sdetN_init"],
            p["detP_init"], p["po4_init"], p["oxy_init"], p["no3_init"], p["nh3_init"],
            p["odu_init"], p["po4_init"]]
    driver.init_concentrations(sed, init)
    # main.F90: bottom water and detritus fluxes (the example sets ODU to pel_O2)
    sed.bdys[0] = run["pel_Temp"]
    sed.bdys[1 + 6] = run["pel_O2"]
    sed.bdys[1 + 7] = run["pel_NO3"]
    sed.bdys[1 + 8] = run["pel_NH4"]
    sed.bdys[1 + 9] = run["pel_O2"]
    sed.bdys[1 + 10] = run["pel_PO4"]
    day = 86400.0
    sed.fluxes[0] = run["pflux_lDetC"] / day
    sed.fluxes[1] = run["pflux_sDetC"] / day
    sed.fluxes[2] = run["pflux_lDetN"] / day
    sed.fluxes[3] = run["pflux_sDetN"] / day
    sed.fluxes[4] = run["pflux_lDetP"] / day
    cs = sed.to_columns()
    cs.dt = run["dt"]
    cs.conc = np.ascontiguousarray(sed.conc)
    return cs
