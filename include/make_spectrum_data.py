"""Generates include/wpbr_spectrum_data.h: the tabulated data of the sampled
spectral representation (CIE 1931 colour matching functions at 1 nm from
360 to 830 nm, and the 32-sample RGB-to-spectrum bases for reflectances and
illuminants), taken as data from the reference's SpectrumData.h, which holds
the same published tables pbrt uses. Literals are copied digit for digit
(double literals in float arrays, as the reference initialises them), so the
float values are identical.

    python include/make_spectrum_data.py <path to SpectrumData.h>
"""
import os
import re
import sys

NAMES = [
    ("CIE_lambda", "kCieLambda", 471), ("CIE_X", "kCieX", 471), ("CIE_Y", "kCieY", 471), ("CIE_Z", "kCieZ", 471),
    ("RGB2SpectLambda", "kRgbLambda", 32),
    ("RGBRefl2SpectWhite", "kReflWhite", 32), ("RGBRefl2SpectCyan", "kReflCyan", 32),
    ("RGBRefl2SpectMagenta", "kReflMagenta", 32), ("RGBRefl2SpectYellow", "kReflYellow", 32),
    ("RGBRefl2SpectRed", "kReflRed", 32), ("RGBRefl2SpectGreen", "kReflGreen", 32),
    ("RGBRefl2SpectBlue", "kReflBlue", 32),
    ("RGBIllum2SpectWhite", "kIllumWhite", 32), ("RGBIllum2SpectCyan", "kIllumCyan", 32),
    ("RGBIllum2SpectMagenta", "kIllumMagenta", 32), ("RGBIllum2SpectYellow", "kIllumYellow", 32),
    ("RGBIllum2SpectRed", "kIllumRed", 32), ("RGBIllum2SpectGreen", "kIllumGreen", 32),
    ("RGBIllum2SpectBlue", "kIllumBlue", 32),
]
NUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?")


def parse(text):
    out = {}
    for src, _, n in NAMES:
        m = re.search(r"const\s+float\s+%s\s*\[[^\]]*\]\s*=\s*\{(.*?)\}" % src, text, re.S)
        if not m:
            raise ValueError("array %s not found" % src)
        body = re.sub(r"//[^\n]*", "", m.group(1))
        vals = NUM.findall(body)
        if len(vals) != n:
            raise ValueError("%s: %d values, expected %d" % (src, len(vals), n))
        out[src] = vals
    return out


def render(tables):
    lines = [
        "/* wpbr_spectrum_data.h — generated by include/make_spectrum_data.py; do not edit.",
        " * Tabulated data of the 64-sample spectral representation: CIE 1931",
        " * colour matching functions (360-830 nm, 1 nm) and the RGB-to-spectrum",
        " * bases (Smits) for reflectances and illuminants, the data the reference's",
        " * SampledSpectrum is built from (SpectrumData.h, CSpectrumSampled.h:216-278). */",
        "#ifndef WPBR_SPECTRUM_DATA_H",
        "#define WPBR_SPECTRUM_DATA_H",
        "",
        "namespace wpbr_spec {",
        "",
        "constexpr int kCieSamples = 471;",
        "constexpr int kRgbSamples = 32;",
        "constexpr int kSpectralSamples = 64;",
        "constexpr unsigned kLambdaStart = 400;",
        "constexpr unsigned kLambdaEnd = 700;",
        "",
    ]
    for src, dst, n in NAMES:
        lines.append("static const float %s[%d] = {" % (dst, n))
        vals = tables[src]
        for i in range(0, n, 6):
            lines.append("    " + ", ".join(vals[i:i + 6]) + ",")
        lines.append("};")
    lines += ["", "}  // namespace wpbr_spec", "", "#endif", ""]
    return "\n".join(lines)


def main(argv):
    src = argv[1] if len(argv) > 1 else os.path.join("/root/reference", "WoodenPBREngine", "SpectrumData.h")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "wpbr_spectrum_data.h")
    with open(src) as f:
        text = f.read()
    with open(out, "w") as f:
        f.write(render(parse(text)))
    print(out)


if __name__ == "__main__":
    main(sys.argv)
