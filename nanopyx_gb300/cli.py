"""Command-line front door: TIFF in, reconstruction or metric out.

The reference's console scripts (src/nanopyx/cli/superresolution.py:10-192,
src/nanopyx/cli/metrics.py:18-145; pyproject.toml:64-74), with the same
functions, arguments, defaults and outputs, computing on the GPU:

    python -m nanopyx_gb300.cli linkinpy-SuperResolution-eSRRF in.tif out.tif --radius 1.5
    python -m nanopyx_gb300.cli linkinpy-SuperResolution-SRRF in.tif out.tif
    python -m nanopyx_gb300.cli linkinpy-Metrics-CalculateErrorMap ref.tif sr.tif map.tif
    python -m nanopyx_gb300.cli linkinpy-Metrics-CalculateFRC a.tif b.tif frc.csv
    python -m nanopyx_gb300.cli linkinpy-Metrics-ImageDecorrelationAnalysis sr.tif dec.csv
"""
from __future__ import annotations

import argparse
import csv
import sys

from .tiff import imread, imwrite


def linkinpy_SRRF(input_image: str, output_image: str, magnification: int = 5,
                  ringRadius: float = 0.5, border: int = 0,
                  radialityPositivityConstraint: bool = True, doIntensityWeighting: bool = True,
                  macro_pixel_correction: bool = True) -> None:
    from .methods import SRRF

    image = imread(input_image)
    output = SRRF(image=image, magnification=magnification, ringRadius=ringRadius, border=border,
                  radialityPositivityConstraint=radialityPositivityConstraint,
                  doIntensityWeighting=doIntensityWeighting,
                  macro_pixel_correction=macro_pixel_correction)
    imwrite(output_image, output)


def _bool(parser, *names, dest, default):
    parser.add_argument(*names, dest=dest, action=argparse.BooleanOptionalAction, default=default)


def linkinpy_SRRF_main(argv=None) -> None:
    parser = argparse.ArgumentParser(description="Run NanoPyx SRRF.")
    parser.add_argument("input_image", help="Input image path.")
    parser.add_argument("output_image", help="Output image path.")
    parser.add_argument("--magnification", type=int, default=5)
    parser.add_argument("--ring-radius", "--ringRadius", dest="ringRadius", type=float,
                        default=0.5)
    parser.add_argument("--border", type=int, default=0)
    _bool(parser, "--radiality-positivity-constraint", "--radialityPositivityConstraint",
          dest="radialityPositivityConstraint", default=True)
    _bool(parser, "--intensity-weighting", "--doIntensityWeighting",
          dest="doIntensityWeighting", default=True)
    _bool(parser, "--macro-pixel-correction", "--macro_pixel_correction",
          dest="macro_pixel_correction", default=True)
    a = parser.parse_args(argv)
    linkinpy_SRRF(a.input_image, a.output_image, a.magnification, a.ringRadius, a.border,
                  a.radialityPositivityConstraint, a.doIntensityWeighting,
                  a.macro_pixel_correction)


def linkinpy_eSRRF(input_image: str, output_image: str, magnification: int = 5,
                   radius: float = 1.5, sensitivity: float = 1.0, frames_per_timepoint: int = 0,
                   temporal_correlation: str = "AVG", use_fht: bool = False,
                   doIntensityWeighting: bool = True, macro_pixel_correction: bool = True,
                   pad_edges: bool = False) -> None:
    from .methods import eSRRF

    image = imread(input_image)
    output = eSRRF(image, magnification=magnification, radius=radius, sensitivity=sensitivity,
                   frames_per_timepoint=frames_per_timepoint,
                   temporal_correlation=temporal_correlation, use_fht=use_fht,
                   doIntensityWeighting=doIntensityWeighting,
                   macro_pixel_correction=macro_pixel_correction, pad_edges=pad_edges)
    imwrite(output_image, output)


def linkinpy_eSRRF_main(argv=None) -> None:
    parser = argparse.ArgumentParser(description="Run NanoPyx eSRRF.")
    parser.add_argument("input_image", help="Input image path.")
    parser.add_argument("output_image", help="Output image path.")
    parser.add_argument("--magnification", type=int, default=5)
    parser.add_argument("--radius", type=float, default=1.5)
    parser.add_argument("--sensitivity", type=float, default=1.0)
    parser.add_argument("--frames-per-timepoint", "--frames_per_timepoint",
                        dest="frames_per_timepoint", type=int, default=0)
    parser.add_argument("--temporal-correlation", "--temporal_correlation",
                        dest="temporal_correlation", default="AVG")
    _bool(parser, "--use-fht", "--use_fht", dest="use_fht", default=False)
    _bool(parser, "--intensity-weighting", "--doIntensityWeighting",
          dest="doIntensityWeighting", default=True)
    _bool(parser, "--macro-pixel-correction", "--macro_pixel_correction",
          dest="macro_pixel_correction", default=True)
    _bool(parser, "--pad-edges", "--pad_edges", dest="pad_edges", default=False)
    a = parser.parse_args(argv)
    linkinpy_eSRRF(a.input_image, a.output_image, a.magnification, a.radius, a.sensitivity,
                   a.frames_per_timepoint, a.temporal_correlation, a.use_fht,
                   a.doIntensityWeighting, a.macro_pixel_correction, a.pad_edges)


# the reference's longer aliases (superresolution.py:148-192)
linkinpy_SuperResolution_SRRF = linkinpy_SRRF
linkinpy_SuperResolution_eSRRF = linkinpy_eSRRF


def _write_scalar_csv(path: str, metric_name: str, value: float) -> None:
    with open(path, "w", newline="", encoding="utf-8") as f:
        w = csv.writer(f)
        w.writerow(["metric", "value"])
        w.writerow([metric_name, float(value)])


def linkinpy_calculate_error_map(input_reference: str, input_super_resolution: str,
                                 output_image: str, output_metrics: str = None) -> None:
    from .scoring import calculate_error_map

    error_map, rse, rsp = calculate_error_map(img_ref=imread(input_reference),
                                              img_sr=imread(input_super_resolution))
    imwrite(output_image, error_map)
    if output_metrics:
        with open(output_metrics, "w", newline="", encoding="utf-8") as f:
            w = csv.writer(f)
            w.writerow(["metric", "value"])
            w.writerow(["RSE", float(rse)])
            w.writerow(["RSP", float(rsp)])


def linkinpy_calculate_error_map_main(argv=None) -> None:
    parser = argparse.ArgumentParser(description="Calculate SQUIRREL error map.")
    parser.add_argument("input_reference", help="Reference image path.")
    parser.add_argument("input_super_resolution", help="Super-resolution image path.")
    parser.add_argument("output_image", help="Output error map image path.")
    parser.add_argument("--output-metrics", "--output_metrics", dest="output_metrics",
                        default=None, help="Optional output CSV path for RSE/RSP.")
    a = parser.parse_args(argv)
    linkinpy_calculate_error_map(a.input_reference, a.input_super_resolution, a.output_image,
                                 a.output_metrics)


def linkinpy_calculate_frc(input_frame_1: str, input_frame_2: str, output_csv: str,
                           pixel_size: float = 1.0, units: str = "pixel",
                           plot_frc_curve: bool = False) -> None:
    from .scoring import calculate_frc

    resolution = calculate_frc(frame_1=imread(input_frame_1), frame_2=imread(input_frame_2),
                               pixel_size=pixel_size, units=units,
                               plot_frc_curve=plot_frc_curve)
    _write_scalar_csv(output_csv, "frc_resolution", float(resolution))


def linkinpy_calculate_frc_main(argv=None) -> None:
    parser = argparse.ArgumentParser(description="Calculate FRC resolution.")
    parser.add_argument("input_frame_1", help="First image path.")
    parser.add_argument("input_frame_2", help="Second image path.")
    parser.add_argument("output_csv", help="Output CSV path.")
    parser.add_argument("--pixel-size", "--pixel_size", dest="pixel_size", type=float,
                        default=1.0)
    parser.add_argument("--units", default="pixel")
    _bool(parser, "--plot-frc-curve", "--plot_frc_curve", dest="plot_frc_curve",
          default=False)
    a = parser.parse_args(argv)
    linkinpy_calculate_frc(a.input_frame_1, a.input_frame_2, a.output_csv, a.pixel_size,
                           a.units, a.plot_frc_curve)


def linkinpy_calculate_decorr_analysis(input_image: str, output_csv: str, rmin: float = 0.0,
                                       rmax: float = 1.0, n_r: int = 50, n_g: int = 10,
                                       pixel_size: float = 1.0, units: str = "pixel",
                                       roi: str = "0,0,0,0",
                                       plot_decorr_analysis: bool = False) -> None:
    from .scoring import calculate_decorr_analysis

    roi_tuple = tuple(int(v.strip()) for v in roi.split(","))
    resolution = calculate_decorr_analysis(frame=imread(input_image), rmin=rmin, rmax=rmax,
                                           n_r=n_r, n_g=n_g, pixel_size=pixel_size,
                                           units=units, roi=roi_tuple,
                                           plot_decorr_analysis=plot_decorr_analysis)
    _write_scalar_csv(output_csv, "decorr_resolution", float(resolution))


def linkinpy_calculate_decorr_analysis_main(argv=None) -> None:
    parser = argparse.ArgumentParser(description="Calculate decorrelation-based resolution.")
    parser.add_argument("input_image", help="Input image path.")
    parser.add_argument("output_csv", help="Output CSV path.")
    parser.add_argument("--rmin", type=float, default=0.0)
    parser.add_argument("--rmax", type=float, default=1.0)
    parser.add_argument("--n-r", "--n_r", dest="n_r", type=int, default=50)
    parser.add_argument("--n-g", "--n_g", dest="n_g", type=int, default=10)
    parser.add_argument("--pixel-size", "--pixel_size", dest="pixel_size", type=float,
                        default=1.0)
    parser.add_argument("--units", default="pixel")
    parser.add_argument("--roi", default="0,0,0,0")
    _bool(parser, "--plot-decorr-analysis", "--plot_decorr_analysis",
          dest="plot_decorr_analysis", default=False)
    a = parser.parse_args(argv)
    linkinpy_calculate_decorr_analysis(a.input_image, a.output_csv, a.rmin, a.rmax, a.n_r,
                                       a.n_g, a.pixel_size, a.units, a.roi,
                                       a.plot_decorr_analysis)


COMMANDS = {
    "linkinpy-SuperResolution-SRRF": linkinpy_SRRF_main,
    "linkinpy-SuperResolution-eSRRF": linkinpy_eSRRF_main,
    "linkinpy-Metrics-CalculateErrorMap": linkinpy_calculate_error_map_main,
    "linkinpy-Metrics-CalculateFRC": linkinpy_calculate_frc_main,
    "linkinpy-Metrics-ImageDecorrelationAnalysis": linkinpy_calculate_decorr_analysis_main,
}


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    if not argv or argv[0] not in COMMANDS:
        print("usage: python -m nanopyx_gb300.cli {" + ",".join(COMMANDS) + "} ...",
              file=sys.stderr)
        return 2
    COMMANDS[argv[0]](argv[1:])
    return 0


if __name__ == "__main__":
    sys.exit(main())
