"""Format parameters used by the oracle (test infrastructure).

The values restate the frozen upstream snapshot the reference embeds
(``src/VHSDecode.Core/Formats/format-params.snapshot.json``, cases
PAL and NTSC, VHS and SVHS, at ``sp``, ``lp`` and ``ep``; read through
``FormatCatalog.cs:46-112``).  VHS LP/EP switch the sub-deemphasis on and
narrow the NTSC RF filters; S-VHS LP/EP equal S-VHS SP.
Only the keys the RF -> TBC luma and chroma paths read are kept.  ``tests/golden/
format_params.json`` (written by ``tests/golden/make_golden.py`` from the
reference snapshot) pins this table.
"""

PAL_VHS_SP = {
    "system": "PAL", "tape_format": "VHS", "tape_speed": "sp",
    "sys": {
        "FPS": 25.0, "ire0": 4100000.0, "hz_ire": 7000.0,
        "vsync_ire": -42.857142857142854, "line_period": 64.0,
        "hsyncPulseUS": 4.7, "eqPulseUS": 2.35, "vsyncPulseUS": 27.3,
        "numPulses": 5, "outlinelen": 1135, "outfreq": 17.734475,
        "frame_lines": 625, "field_lines": [312, 313], "outputZero": 256,
        "fsc_mhz": 4.43361875, "colorBurstUS": [5.6, 7.85], "burst_abs_ref": 5000,
    },
    "rf": {
        "video_bpf_low": 1300000.0, "video_bpf_high": 5780000.0,
        "video_bpf_order": None, "video_bpf_supergauss": False,
        "video_lpf_extra": 5910000.0, "video_lpf_extra_order": 20,
        "video_hpf_extra": 1320000.0, "video_hpf_extra_order": 12,
        "video_rf_peak_freq": 4300000.0, "video_rf_peak_gain": 4.0,
        "video_rf_peak_bandwidth": 10000000.0,
        "boost_rf_linear_0": 0.0, "boost_rf_linear_20": 1.0,
        "start_rf_linear": 626953.0, "boost_rf_linear_double": False,
        "video_lpf_freq": 3400000.0, "video_lpf_order": 6,
        "video_lpf_supergauss": False,
        "deemph_gain": 13.9794, "deemph_mid": 273755.82,
        "deemph_q": 0.462088186,
        "color_under_carrier": 626953.0,
        "chroma_bpf_upper": 1300000, "chroma_rotation": [0, -1],
    },
}

NTSC_VHS_SP = {
    "system": "NTSC", "tape_format": "VHS", "tape_speed": "sp",
    "sys": {
        "FPS": 29.970029970029973, "ire0": 3685714.2857142854,
        "hz_ire": 7142.857142857143, "vsync_ire": -40.0,
        "line_period": 63.55555555555555, "hsyncPulseUS": 4.7,
        "eqPulseUS": 2.3, "vsyncPulseUS": 27.1, "numPulses": 6,
        "outlinelen": 910, "outfreq": 14.318181818181818,
        "frame_lines": 525, "field_lines": [263, 262], "outputZero": 1024,
        "fsc_mhz": 3.5795454545454546, "colorBurstUS": [5.3, 7.8], "burst_abs_ref": 4416,
    },
    "rf": {
        "video_bpf_low": 500000.0, "video_bpf_high": 6500000.0,
        "video_bpf_order": 8, "video_bpf_supergauss": False,
        "video_lpf_extra": 6000000.0, "video_lpf_extra_order": 25,
        "video_hpf_extra": 1200000.0, "video_hpf_extra_order": 20,
        "video_rf_peak_freq": 3900000.0, "video_rf_peak_gain": 4.0,
        "video_rf_peak_bandwidth": 10000000.0,
        "boost_rf_linear_0": 0.0, "boost_rf_linear_20": 1.0,
        "start_rf_linear": 629370.6293706294, "boost_rf_linear_double": False,
        "video_lpf_freq": 6600000.0, "video_lpf_order": 9,
        "video_lpf_supergauss": True,
        "deemph_gain": 13.9794, "deemph_mid": 273755.82,
        "deemph_q": 0.462088186,
        "color_under_carrier": 629370.6293706294,
        "chroma_bpf_upper": 1200000, "chroma_rotation": [-1, 1],
    },
}

_SVHS_RF = {
    "video_bpf_low": 2000000.0, "video_bpf_high": 8980000.0,
    "video_bpf_order": None, "video_bpf_supergauss": False,
    "video_lpf_extra": 9100000.0, "video_lpf_extra_order": 25,
    "video_hpf_extra": 1300000.0, "video_hpf_extra_order": 20,
    "video_rf_peak_freq": 6200000.0, "video_rf_peak_gain": 4.0,
    "video_rf_peak_bandwidth": 16000000.0,
    "boost_rf_linear_0": 1.0, "boost_rf_linear_20": 4.0,
    "video_lpf_freq": 7500000.0, "video_lpf_order": 6, "video_lpf_supergauss": True,
    "video_custom_luma_filters": [
        {"type": "file", "filename": "svhs-sp-linear-subdeemphasis"},
        {"type": "highshelf", "midfreq": 2000000.0, "gain": 4.0, "q": 0.4967045}],
    "use_sub_deemphasis": True,
    "nonlinear_highpass_freq": 320000.0, "nonlinear_amp_lpf_freq": 590000.0,
    "nonlinear_exp_scaling": 0.23, "nonlinear_scaling_1": None, "nonlinear_scaling_2": 0.72,
    "nonlinear_logistic_mid": 0.2, "nonlinear_logistic_rate": 14.0,
}


def _svhs(base, ire0, hz_ire):
    fmt = {"system": base["system"], "tape_format": "SVHS", "tape_speed": "sp",
           "sys": dict(base["sys"], ire0=ire0, hz_ire=hz_ire), "rf": dict(base["rf"])}
    fmt["rf"].update(_SVHS_RF)
    return fmt


PAL_SVHS_SP = _svhs(PAL_VHS_SP, 5880000.0, 11200.0)
NTSC_SVHS_SP = _svhs(NTSC_VHS_SP, 5857142.857142857, 11428.57142857143)

_VHS_LONG_PLAY_RF = {
    "use_sub_deemphasis": True, "nonlinear_highpass_freq": 820000.0,
    "nonlinear_exp_scaling": 0.12, "nonlinear_scaling_1": 0.1,
}


def _long_play(base, speed, ntsc_lpf_extra=None, ntsc_bpf_high=None, burst_abs_ref=None):
    fmt = {"system": base["system"], "tape_format": base["tape_format"], "tape_speed": speed,
           "sys": dict(base["sys"]), "rf": dict(base["rf"])}
    if burst_abs_ref is not None:
        fmt["sys"]["burst_abs_ref"] = burst_abs_ref
    if base["tape_format"] == "VHS":
        fmt["rf"].update(_VHS_LONG_PLAY_RF)
        if ntsc_lpf_extra is not None:
            fmt["rf"]["video_lpf_extra"] = ntsc_lpf_extra
        if ntsc_bpf_high is not None:
            fmt["rf"]["video_bpf_high"] = ntsc_bpf_high
    return fmt


FORMATS = {("PAL", "VHS", "sp"): PAL_VHS_SP, ("NTSC", "VHS", "sp"): NTSC_VHS_SP,
           ("PAL", "SVHS", "sp"): PAL_SVHS_SP, ("NTSC", "SVHS", "sp"): NTSC_SVHS_SP,
           ("PAL", "VHS", "lp"): _long_play(PAL_VHS_SP, "lp"),
           ("PAL", "VHS", "ep"): _long_play(PAL_VHS_SP, "ep"),
           ("NTSC", "VHS", "lp"): _long_play(NTSC_VHS_SP, "lp", 5900000.0, burst_abs_ref=2208.0),
           ("NTSC", "VHS", "ep"): _long_play(NTSC_VHS_SP, "ep", 5800000.0, 6400000.0),
           ("PAL", "SVHS", "lp"): _long_play(PAL_SVHS_SP, "lp"),
           ("PAL", "SVHS", "ep"): _long_play(PAL_SVHS_SP, "ep"),
           ("NTSC", "SVHS", "lp"): _long_play(NTSC_SVHS_SP, "lp"),
           ("NTSC", "SVHS", "ep"): _long_play(NTSC_SVHS_SP, "ep")}


def get(system: str, tape_format: str = "VHS", speed: str = "sp") -> dict:
    return FORMATS[(system.upper(), tape_format.upper(), speed.lower())]


def sub_deemphasis(fmt: dict):
    """``DecodeSession.BuildSubDeemphasisOptions`` (Core/Decode/DecodeSession.cs:1250-1278),
    or None when the format does not use sub-deemphasis."""
    rf, sy = fmt["rf"], fmt["sys"]
    if not rf.get("use_sub_deemphasis"):
        return None
    dev = sy.get("nonlinear_deviation")
    if dev is None:
        dev = sy["hz_ire"] * (100.0 + -sy["vsync_ire"])
    return {"highpass": rf["nonlinear_highpass_freq"],
            "bandpass_upper": rf.get("nonlinear_bandpass_upper"),
            "order": rf.get("nonlinear_bandpass_order") or 1,
            "amp_lpf": rf.get("nonlinear_amp_lpf_freq") or 700000.0,
            "deviation": dev,
            "exp": rf.get("nonlinear_exp_scaling") if rf.get("nonlinear_exp_scaling") is not None else 0.25,
            "scale1": rf.get("nonlinear_scaling_1"), "scale2": rf.get("nonlinear_scaling_2"),
            "logistic_mid": rf.get("nonlinear_logistic_mid"),
            "logistic_rate": rf.get("nonlinear_logistic_rate"),
            "static": rf.get("nonlinear_static_factor")}


def output_scale(fmt: dict) -> float:
    """``VideoOutputConverter.ComputeOutputScale`` (Core/Tbc/VideoOutputConverter.cs:129-138)."""
    dividend = (0xD300 - 0x0100) if fmt["system"] == "PAL" else (0xC800 - 0x0400)
    return dividend / (100.0 - fmt["sys"]["vsync_ire"])
