"""ctypes binding of libgomelt.so (declared in include/gomelt.h).

The library is the only compute path: if it is missing or fails to load, every
call raises ``GomeltError``; there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgomelt.so")

GM_OK, GM_ERR_ARG, GM_ERR_LAUNCH, GM_ERR_CUDA, GM_ERR_UNSUPPORTED, GM_ERR_TOO_LARGE = range(6)
GM_F32, GM_F64 = 0, 1
_ERRNAMES = {1: "invalid argument", 2: "kernel launch failed", 3: "CUDA runtime error",
             4: "unsupported configuration", 5: "request exceeds a fixed capacity"}


class GomeltError(RuntimeError):
    pass


vp = C.c_void_p


class gm_props(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "k_powder", "k_bulk_a0", "k_bulk_a1", "k_fluid",
        "cp_solid_a0", "cp_solid_a1", "cp_mushy", "cp_fluid", "rho",
        "T_amb", "T_solidus", "T_liquidus", "T_boiling",
        "h_conv", "emissivity", "sigma_sb", "evc", "Lev", "CM_coeff", "CT_coeff", "CP_coeff",
        "laser_radius", "laser_depth", "laser_eta")]


class gm_map3(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("src_nx", C.c_int), ("src_ny", C.c_int),
                ("elem", vp * 3), ("w", vp * 3)]


class gm_level_args(C.Structure):
    _fields_ = [
        ("dtype", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("h", C.c_double * 3), ("origin", C.c_double * 3), ("ne_planes", C.c_int),
        ("dt", vp), ("T_in", vp), ("T_out", vp), ("ph_in", vp), ("ph_out", vp),
        ("substrate", C.c_longlong), ("k_arr", vp), ("rc_arr", vp), ("F_full", vp), ("corr_full", vp),
        ("rhs_box", vp), ("box", C.c_int * 6), ("laser", vp), ("surface", C.c_int), ("bc_mode", C.c_int),
        ("face", C.c_double * 5), ("inactive_amb", C.c_int), ("bc_new", vp), ("bc_old", vp),
        ("bc_alpha", C.c_double), ("bc_beta", C.c_double), ("bc_map", gm_map3), ("clamp", C.c_int),
        ("accum", vp), ("max_accum", vp), ("zchunk", C.c_int), ("pdl", C.c_int), ("src_tab", vp),
        ("status", vp),
    ]


class gm_ring_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("nodes", C.c_int * 3), ("map", gm_map3), ("srcA", vp), ("srcB", vp),
                ("outA", vp), ("outB", vp)]


class gm_energy_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("nodes", C.c_int * 3), ("h", C.c_double * 3), ("origin", C.c_double * 3),
                ("ne_planes", C.c_int), ("T0", vp), ("T1", vp), ("ph", vp), ("substrate", C.c_longlong),
                ("interval", C.c_double), ("rows", vp), ("npos", C.c_int), ("scratch", vp),
                ("scratch_cap", C.c_longlong), ("out", vp)]


class gm_meltpool_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("nodes", C.c_int * 3), ("h", C.c_double * 3), ("origin", C.c_double * 3),
                ("T", vp), ("iso", C.c_double), ("scratch", vp), ("scratch_cap", C.c_longlong), ("out", vp)]


class gm_conv_args(C.Structure):
    _fields_ = [("grid", C.c_int * 4), ("cin", C.c_int), ("cout", C.c_int), ("in_", vp), ("in_stride", C.c_int),
                ("in_off", C.c_int), ("w", vp), ("bias", vp), ("relu", C.c_int), ("mask", vp),
                ("mask_stride", C.c_int), ("mask_off", C.c_int), ("mirror", C.c_int), ("out", vp),
                ("out_stride", C.c_int), ("out_off", C.c_int), ("wpack", vp)]


class gm_wgrad_args(C.Structure):
    _fields_ = [("grid", C.c_int * 4), ("cin", C.c_int), ("cout", C.c_int), ("in_", vp), ("in_stride", C.c_int),
                ("in_off", C.c_int), ("dy", vp), ("dy_stride", C.c_int), ("dy_off", C.c_int), ("dw", vp),
                ("scratch", vp), ("scratch_cap", C.c_longlong)]


class gm_adam_args(C.Structure):
    _fields_ = [("n", C.c_longlong), ("w", vp), ("grad", vp), ("m", vp), ("v", vp), ("lr", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float), ("c1", C.c_float),
                ("c2", C.c_float), ("wd", C.c_float), ("wb", vp), ("wt", vp), ("cout", C.c_int), ("cin", C.c_int)]


class gm_surr_args(C.Structure):
    _fields_ = [("grid", C.c_int * 4), ("nodes", C.c_int * 3), ("T2i", vp), ("T3o", vp), ("T3n", vp), ("par", vp),
                ("T_amb", C.c_double), ("scale", C.c_double), ("x", vp), ("target", vp), ("lmask", vp)]


class gm_batch_info(C.Structure):
    _fields_ = [("nb", C.c_int), ("dtype", C.c_int), ("variant", C.c_int), ("blocks", C.c_int),
                ("kernel", C.c_int), ("rows", C.c_int), ("warps", C.c_int)]


class gm_tune_result(C.Structure):
    _fields_ = [("tile_x", C.c_int), ("tile_y", C.c_int), ("zchunk", C.c_int), ("us", C.c_float),
                ("kernel", C.c_int), ("rows", C.c_int)]


class gm_level_shape(C.Structure):
    _fields_ = [("kernel", C.c_int), ("tile_x", C.c_int), ("tile_y", C.c_int), ("rows", C.c_int),
                ("zchunk", C.c_int)]


class gm_state_props_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_longlong), ("T", vp), ("ph_in", C.POINTER(C.c_uint8)),
                ("ph_out", C.POINTER(C.c_uint8)), ("k_out", vp), ("rc_out", vp), ("substrate", C.c_longlong)]


class gm_interp_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_int * 3), ("nterms", C.c_int), ("map", gm_map3 * 3),
                ("src", vp * 3), ("coef", C.c_double * 3), ("base", vp), ("out", vp), ("out_term", vp),
                ("which_term", C.c_int)]


class gm_restrict_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_int * 3), ("map", gm_map3), ("cidx", C.POINTER(C.c_int) * 3),
                ("cnx", C.c_int), ("cny", C.c_int), ("fine", vp), ("coarse", vp)]


class gm_tprime_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_int * 3), ("cmap", gm_map3), ("cf0", C.POINTER(C.c_int) * 3),
                ("cf1", C.POINTER(C.c_int) * 3), ("c_of_f", C.POINTER(C.c_int) * 3), ("cnx", C.c_int),
                ("cny", C.c_int), ("fine", vp), ("coarse", vp), ("out", vp)]


class gm_restrict_s1_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_int * 3), ("map", gm_map3), ("cidx", C.POINTER(C.c_int) * 3),
                ("cnx", C.c_int), ("cny", C.c_int), ("fine_ph", C.POINTER(C.c_uint8)),
                ("coarse_ph", C.POINTER(C.c_uint8)), ("substrate", C.c_longlong)]


class gm_l0_args(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("idx", C.POINTER(C.c_int) * 3), ("l0_nx", C.c_longlong),
                ("l0_ny", C.c_longlong), ("l0_bits", vp), ("ph", C.POINTER(C.c_uint8)),
                ("prev_ph", C.POINTER(C.c_uint8)), ("prev_lo", C.c_int * 3), ("prev_n", C.c_int * 3)]


class gm_couple_axis(C.Structure):
    _fields_ = [("nfe", C.c_int), ("cw", vp), ("node0", C.POINTER(C.c_int)), ("cb_lo", C.c_int),
                ("ncb", C.c_int), ("flo", C.POINTER(C.c_int)), ("fhi", C.POINTER(C.c_int)), ("rmax", C.c_int),
                ("H", C.c_double)]


class gm_couple_geom(C.Structure):
    _fields_ = [("ax", gm_couple_axis * 3)]


class gm_couple_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("geom", gm_couple_geom), ("fine_nodes", C.c_int * 3),
                ("fine_h", C.c_double * 3), ("T", vp), ("ph", C.POINTER(C.c_uint8)), ("substrate", C.c_longlong),
                ("k_arr", vp), ("rc_arr", vp), ("Tp", vp), ("dTa", vp), ("dTb", vp), ("dt", vp), ("out", vp),
                ("out_lo", C.c_int * 3), ("out_n", C.c_int * 3), ("scale", C.c_double), ("partials", vp),
                ("partials_cap", C.c_longlong), ("method", C.c_int), ("base", vp)]


class gm_coarse_source_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("geom", gm_couple_geom), ("npos", C.c_int), ("rows", vp),
                ("xq", C.POINTER(C.c_double) * 3), ("fine_wq", C.c_double), ("out", vp), ("out_lo", C.c_int * 3),
                ("out_n", C.c_int * 3), ("scratch", vp), ("scratch_cap", C.c_longlong), ("ngroups", C.c_int),
                ("out_group_stride", C.c_longlong)]


class gm_window(C.Structure):
    _fields_ = [("nodes", C.c_int * 3), ("h", C.c_double * 3), ("origin", C.c_double * 3),
                ("substrate", C.c_longlong), ("T", vp), ("Tp", vp), ("ph", C.POINTER(C.c_uint8))]


_P_INT = C.POINTER(C.c_int)
_P_DBL = C.POINTER(C.c_double)
_P_U8 = C.POINTER(C.c_uint8)


class gm_subcycle_plan(C.Structure):
    _fields_ = [
        ("dtype", C.c_int), ("N2", C.c_int), ("N3", C.c_int), ("L1", gm_window), ("L2", gm_window),
        ("L3", gm_window), ("L1_ne_planes", C.c_int), ("face", C.c_double * 5), ("acc3", vp), ("macc3", vp),
        ("bc12", gm_map3), ("bc23", gm_map3), ("r32", gm_map3), ("r21", gm_map3), ("r32_idx", _P_INT * 3),
        ("r21_idx", _P_INT * 3), ("c32", gm_couple_geom), ("c31", gm_couple_geom), ("c21", gm_couple_geom),
        ("xq32", _P_DBL * 3), ("xq31", _P_DBL * 3), ("rhs1_lo", C.c_int * 3), ("rhs1_n", C.c_int * 3),
        ("rhs2_lo", C.c_int * 3), ("rhs2_n", C.c_int * 3), ("L0", vp), ("L0_nx", C.c_longlong),
        ("L0_ny", C.c_longlong), ("l0_idx3", _P_INT * 3), ("rows", vp), ("dts", vp), ("T1p", vp), ("T1c", vp),
        ("T2w", vp * 2), ("T3w", vp * 2), ("tp3w", vp * 2), ("Tp2w", vp), ("rhs1", vp), ("rhs2", vp),
        ("tp3hist", vp), ("ph2w", _P_U8 * 2), ("ph3w", _P_U8 * 2), ("partials", vp), ("partials_cap", C.c_longlong),
        ("src_scratch", vp), ("src_cap", C.c_longlong), ("src2", vp), ("L2all", vp), ("L3all", vp), ("L3pall", vp),
        ("zchunk", C.c_int), ("ring2", vp * 2), ("ring3", vp * 2), ("graph", C.c_int),
        ("pdl", C.c_int), ("src3tab", vp), ("persist", C.c_int), ("xch3", vp * 2), ("pflags", vp),
        ("pflags_cap", C.c_longlong), ("pstatus", vp), ("inj32", C.POINTER(C.c_int) * 9),
        ("inj21", C.POINTER(C.c_int) * 9), ("l3_pairs", C.c_int)]


class gm_persist_args(C.Structure):
    _fields_ = [("dtype", C.c_int), ("nodes", C.c_int * 3), ("h", C.c_double * 3), ("nsteps", C.c_int),
                ("nsub", C.c_int), ("T_in", vp), ("T_out", vp), ("ph_in", vp), ("ph_out", vp),
                ("substrate", C.c_longlong), ("ring_new", vp), ("ring_old", vp), ("src_tab", vp), ("rows", vp),
                ("accum", vp), ("max_accum", vp), ("xbuf", vp * 2), ("flags", vp), ("flags_cap", C.c_longlong),
                ("base", C.c_uint), ("status", vp), ("hold", C.c_int)]


GM_PERSIST_TIMEOUT, GM_PERSIST_BAD_T = 1, 2
GM_STATUS_BAD_T = GM_PERSIST_BAD_T


class gm_steps_args(C.Structure):
    _fields_ = [("level", gm_level_args), ("nsteps", C.c_int), ("nsub", C.c_int), ("rows", vp), ("src_tab", vp),
                ("tbuf", vp * 2), ("counter", vp), ("base", C.c_uint), ("status", vp)]


class gm_level2_args(C.Structure):
    _fields_ = [("level", gm_level_args), ("dt2", vp), ("src_tab2", vp), ("bc_alpha2", C.c_double),
                ("bc_beta2", C.c_double)]


class gm_toolpath_state(C.Structure):
    _fields_ = [("run", C.c_longlong), ("k", C.c_longlong), ("row", C.c_longlong), ("x", C.c_double),
                ("y", C.c_double), ("t", C.c_double)]


def subcycle_kernel_count(N2: int, N3: int, separable: bool = False, persist: bool = False,
                          inject32: bool = False, inject21: bool = False, pairs: bool = False) -> int:
    """Kernels gm_subcycle launches: the N2 Level-2 sources (2), set-up and
    Level 1 (8), two passes of a Level-2 ring prolongation plus N2 Level-2
    steps (coupling 2 onto the step's source, Level-2 solve, Level-3 ring, N3
    Level-3 solves, restriction, T'), the T'2/mass/corrector block (7) and the tail
    (3).  For a constant-property material (separable kernels) each of the
    4 + 2 N2 coupling calls is one kernel more and the Level-3 laser factors
    are tabulated once (one kernel).  With persistent Level-3 steps the N3
    solves of a Level-2 step are one kernel; with paired Level-3 steps
    (gm_level_step2) they are N3 // 2 + N3 % 2.  Where a restriction is an
    injection its restriction and T' are one kernel (inject32: the 2 N2
    Level-3 ones, inject21: the two Level-2 ones)."""
    n3 = 1 if persist else (N3 // 2 + N3 % 2 if pairs else N3)
    n = 20 + 2 * (1 + N2 * (6 + n3))
    n -= (2 * N2 if inject32 else 0) + (2 if inject21 else 0)
    return n + (4 + 2 * N2 + 1 if separable else 0)


def props_constant(s) -> bool:
    """k and rho*cp of a gm_props independent of phase and temperature (the
    condition under which the library takes its separable level-step and
    coupling kernels)."""
    return (s.k_powder == s.k_bulk_a0 and s.k_fluid == s.k_bulk_a0 and s.k_bulk_a1 == 0.0 and
            s.cp_solid_a1 == 0.0 and s.cp_mushy == s.cp_solid_a0 and s.cp_fluid == s.cp_solid_a0)


_lib = None


def lib():
    """Load libgomelt.so once; raise GomeltError if it is not there."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GomeltError(f"{LIB_PATH} not found: build it with build_lib.build() (nvcc, sm_103a)")
        try:
            L = C.CDLL(LIB_PATH)
        except OSError as e:
            raise GomeltError(f"cannot load {LIB_PATH}: {e}") from e
        L.gm_version.restype = C.c_char_p
        for name, args in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.gm_couple_partials_size.argtypes = [C.POINTER(gm_couple_geom)]
        L.gm_couple_partials_size.restype = C.c_longlong
        L.gm_level_batched_desc_size.argtypes = [C.c_int, C.c_int]
        L.gm_level_batched_desc_size.restype = C.c_longlong
        L.gm_diag_scratch_size.argtypes = [C.c_int]
        L.gm_diag_scratch_size.restype = C.c_longlong
        L.gm_unet_wgrad_scratch.argtypes = [C.POINTER(C.c_int), C.c_int, C.c_int]
        L.gm_unet_wgrad_scratch.restype = C.c_longlong
        L.gm_unet_head_scratch.argtypes = [C.c_longlong, C.c_int]
        L.gm_unet_head_scratch.restype = C.c_longlong
        L.gm_level3_persist_flags.argtypes = [C.POINTER(C.c_int)]
        L.gm_level3_persist_flags.restype = C.c_longlong
        L.gm_l0_words.argtypes = [C.c_longlong, C.c_longlong, C.c_longlong]
        L.gm_l0_words.restype = C.c_longlong
        _lib = L
    return _lib


SIGNATURES = {
    "gm_level_step": [C.POINTER(gm_level_args), C.POINTER(gm_props), vp],
    "gm_level3_persist": [C.POINTER(gm_persist_args), C.POINTER(gm_props), vp],
    "gm_level3_steps": [C.POINTER(gm_steps_args), C.POINTER(gm_props), vp],
    "gm_toolpath_rows": [vp, C.c_int, vp, C.c_int, C.c_int, vp, vp, vp],
    "gm_l0_fill": [vp, C.c_longlong, C.c_longlong, C.c_longlong, C.c_longlong, C.c_longlong, C.c_int, vp],
    "gm_level3_persist_shape": [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "gm_state_properties": [C.POINTER(gm_state_props_args), C.POINTER(gm_props), vp],
    "gm_fine_source": [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double), vp,
                       C.POINTER(gm_props), vp, vp],
    "gm_surface_flux": [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int, vp, C.POINTER(gm_props),
                        vp, vp],
    "gm_clamp_min": [C.c_int, vp, C.c_longlong, C.c_double, vp],
    "gm_interp": [C.POINTER(gm_interp_args), vp],
    "gm_interp_matrix": [C.c_int, C.POINTER(gm_map3), vp, vp, vp],
    "gm_interp_w_matrix": [C.c_int, vp, vp, vp, vp, C.c_longlong, vp],
    "gm_restrict": [C.POINTER(gm_restrict_args), vp],
    "gm_tprime_inject": [C.POINTER(gm_tprime_args), vp],
    "gm_restrict_s1": [C.POINTER(gm_restrict_s1_args), vp],
    "gm_l0_gather": [C.POINTER(gm_l0_args), vp],
    "gm_l0_scatter": [C.POINTER(gm_l0_args), vp],
    "gm_couple": [C.POINTER(gm_couple_args), C.POINTER(gm_props), vp],
    "gm_coarse_source": [C.POINTER(gm_coarse_source_args), C.POINTER(gm_props), vp],
    "gm_subcycle": [C.POINTER(gm_subcycle_plan), C.POINTER(gm_props), vp],
    "gm_subcycle_batched": [C.POINTER(gm_subcycle_plan), C.c_int, C.POINTER(gm_props), vp],
    "gm_ring_prolong": [C.POINTER(gm_ring_args), vp],
    "gm_level_step_batched": [vp, C.c_int, vp, vp, C.c_longlong, vp],
    "gm_level_batched_prepare": [vp, C.c_int, vp, vp, C.c_longlong, C.POINTER(gm_batch_info), vp],
    "gm_level_batched_launch": [vp, C.POINTER(gm_batch_info), vp],
    "gm_level_autotune": [C.POINTER(gm_level_args), C.POINTER(gm_props), C.c_int, C.POINTER(gm_tune_result), vp],
    "gm_level_step_shape": [C.POINTER(gm_level_args), C.POINTER(gm_props), C.POINTER(gm_level_shape), vp],
    "gm_level_step2": [C.POINTER(gm_level2_args), C.POINTER(gm_props), vp],
    "gm_level_step2_shape": [C.POINTER(gm_level2_args), C.POINTER(gm_props), C.POINTER(gm_level_shape), vp],
    "gm_level_autotune2": [C.POINTER(gm_level2_args), C.POINTER(gm_props), C.c_int, C.POINTER(gm_tune_result),
                           vp],
    "gm_fine_source_tables": [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double), vp,
                              C.c_int, C.POINTER(gm_props), vp, vp],
    "gm_energy_balance": [C.POINTER(gm_energy_args), C.POINTER(gm_props), vp],
    "gm_melt_pool": [C.POINTER(gm_meltpool_args), vp],
    "gm_field_error": [C.c_int, vp, C.c_int, vp, C.c_longlong, vp, C.c_longlong, vp, vp],
    "gm_unet_conv3": [C.POINTER(gm_conv_args), vp],
    "gm_unet_conv3_tc": [C.POINTER(gm_conv_args), vp],
    "gm_unet_conv3_mma": [C.POINTER(gm_conv_args), vp],
    "gm_unet_conv3_tc_eligible": [C.POINTER(gm_conv_args)],
    "gm_unet_tc_status": [],
    "gm_unet_wgrad": [C.POINTER(gm_wgrad_args), vp],
    "gm_unet_bias_grad": [C.POINTER(C.c_int), C.c_int, vp, C.c_int, C.c_int, vp, C.c_longlong, vp, vp],
    "gm_unet_pool2": [C.POINTER(C.c_int), C.c_int, vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp],
    "gm_unet_up2": [C.POINTER(C.c_int), C.c_int, vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, C.c_int, vp],
    "gm_unet_add_slice": [C.c_longlong, C.c_int, vp, C.c_int, C.c_int, vp, C.c_int, C.c_int, vp, C.c_int, C.c_int,
                          vp],
    "gm_unet_head": [C.c_longlong, C.c_int, vp, C.c_int, C.c_int, vp, C.c_float, vp, vp],
    "gm_unet_head_bwd": [C.c_longlong, C.c_int, vp, C.c_int, C.c_int, vp, vp, vp, vp, C.c_float, vp, C.c_int,
                         C.c_int, vp, C.c_longlong, vp, vp],
    "gm_unet_adam": [C.POINTER(gm_adam_args), vp],
    "gm_surrogate_pack": [C.POINTER(gm_surr_args), vp],
    "gm_surrogate_unpack": [C.POINTER(gm_surr_args), vp, vp, vp],
    "gm_couple_noalloc": [C.POINTER(gm_couple_args), C.POINTER(gm_props), vp],
}


def check(code: int, what: str):
    if code != GM_OK:
        raise GomeltError(f"{what}: {_ERRNAMES.get(code, code)}")


# kernels launched by each entry point (for launch accounting)
KERNELS_PER_CALL = {"gm_couple": 2, "gm_coarse_source": 2, "gm_unet_wgrad": 2, "gm_unet_bias_grad": 2,
                    "gm_unet_head_bwd": 2, "gm_level_batched_prepare": 0}
_launches = [0]


def reset_launch_count():
    _launches[0] = 0


def launch_count() -> int:
    return _launches[0]


def call(name: str, *args, kernels=None):
    check(getattr(lib(), name)(*args), name)
    _launches[0] += kernels if kernels is not None else KERNELS_PER_CALL.get(name, 1)


def props_struct(p: dict) -> gm_props:
    """gm_props from a SetupProperties-style dict."""
    s = gm_props()
    s.k_powder = float(p["k_powder"])
    s.k_bulk_a0 = float(p["k_bulk_coeff_a0"])
    s.k_bulk_a1 = float(p["k_bulk_coeff_a1"])
    s.k_fluid = float(p["k_fluid_coeff_a0"])
    s.cp_solid_a0 = float(p["cp_solid_coeff_a0"])
    s.cp_solid_a1 = float(p["cp_solid_coeff_a1"])
    s.cp_mushy = float(p["cp_mushy"])
    s.cp_fluid = float(p["cp_fluid"])
    s.rho = float(p["rho"])
    s.T_amb = float(p["T_amb"])
    s.T_solidus = float(p["T_solidus"])
    s.T_liquidus = float(p["T_liquidus"])
    s.T_boiling = float(p["T_boiling"])
    s.h_conv = float(p["h_conv"])
    s.emissivity = float(p["vareps"])
    s.sigma_sb = float(p["sigma_sb"])
    s.evc = float(p["evc"])
    s.Lev = float(p["Lev"])
    s.CM_coeff = float(p["CM_coeff"])
    s.CT_coeff = float(p["CT_coeff"])
    s.CP_coeff = float(p["CP_coeff"])
    s.laser_radius = float(p["laser_radius"])
    s.laser_depth = float(p["laser_depth"])
    s.laser_eta = float(p["laser_eta"])
    return s
