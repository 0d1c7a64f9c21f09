"""stereo_img's parameter / config-file interface (stereo/stereo_img.cpp:47-103).

Options, types and defaults are the reference's.  A config file holds
`key = value` lines (boost::program_options::parse_config_file syntax, '#'
starts a comment); values given on the command line win over the file,
because the reference stores the command line first and boost keeps the
first stored value (stereo/stereo_img.cpp:94-103).
"""

OPTIONS = {
    # general (stereo/stereo_img.cpp:47-64)
    "im0": (str, None), "im1": (str, None),
    "disp-min": (float, 1.0), "disp-step": (float, 1.0), "disp-max": (float, 128.0),
    "matching": (str, "CENSUS"), "volume": (str, ""), "inference": (str, "CRF"),
    "refinement": (str, "NONE"), "alpha": (float, 20.0), "beta": (float, 0.8),
    "gpu": (int, 0), "output-file": (str, "./output"), "config-file": (str, None),
    # CNN (:65-70)
    "num-layers": (int, 7), "parameter-file": (str, "params"), "with-xy": (bool, False),
    # CENSUS (:71-74)
    "filter-size": (int, 7),
    # CRF (:75-82)
    "lambda": (float, 0.4), "L1": (float, 1.0), "L2": (float, 12.0), "delta": (float, 2.0),
    "crf-iterations": (int, 4),
    # refinement (:83-87)
    "ref-iterations": (int, 10), "warps": (int, 2),
}
SHORT = {"g": "gpu", "o": "output-file"}
MATCHING = ("CENSUS", "COLORCNN", "COLORPAIR", "LOAD")
INFERENCE = ("CRF", "ARGMAX", "NONE")
REFINEMENT = ("NONE", "THuberQuad", "QuadDirect")


def _convert(key, value):
    if key not in OPTIONS:
        raise KeyError("unrecognised option '%s'" % key)
    typ = OPTIONS[key][0]
    if typ is bool:
        v = str(value).strip().lower()
        if v in ("1", "true", "yes", "on"):
            return True
        if v in ("0", "false", "no", "off"):
            return False
        raise ValueError("bad boolean for %s: %r" % (key, value))
    return typ(value)


def parse_cfg_text(text):
    out = {}
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if "=" not in line:
            raise ValueError("config line without '=': %r" % raw)
        k, v = (s.strip() for s in line.split("=", 1))
        if k not in out:  # first value wins, as boost stores it
            out[k] = _convert(k, v)
    return out


def parse_argv(argv, positional=None):
    out, pos = {}, list(positional or [])
    i = 0
    while i < len(argv):
        a = argv[i]
        if a.startswith("--"):
            key, _, val = a[2:].partition("=")
            if not _ and key in OPTIONS:
                if OPTIONS[key][0] is bool and (i + 1 >= len(argv) or argv[i + 1].startswith("-")):
                    val = "true"
                else:
                    i += 1
                    val = argv[i]
            out.setdefault(key, _convert(key, val))
        elif a.startswith("-") and len(a) == 2 and a[1] in SHORT:
            i += 1
            out.setdefault(SHORT[a[1]], _convert(SHORT[a[1]], argv[i]))
        else:
            pos.append(a)
        i += 1
    for key, v in zip(("im0", "im1"), pos):
        out.setdefault(key, v)
    return out


def resolve(argv, cfg_text=None, positional=None):
    """Command line, then the config file, then the reference defaults."""
    cli = parse_argv(argv, positional)
    cfg = {}
    if cfg_text is not None:
        cfg = parse_cfg_text(cfg_text)
    elif cli.get("config-file"):
        try:
            with open(cli["config-file"]) as f:
                cfg = parse_cfg_text(f.read())
        except OSError:
            cfg = {}  # the reference silently ignores an unreadable file (ifs.good())
    full = {k: d for k, (_, d) in OPTIONS.items()}
    full.update(cfg)
    full.update(cli)
    return full
