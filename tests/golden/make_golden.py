"""Extracts MOCC's own known-answer data for the ray tracer into a fixture.

Reads (as text) the reference test sources and their geometry inputs:
  src/sweepers/moc/tests/test_Ray.cpp      weird_ray golden segments,
                                           simple_ray / big_ray coarse data
  src/sweepers/moc/tests/6x5.xml, large.xml, square.xml (geometries)
  src/sweepers/moc/tests/test_RayData.cpp  volume-conservation test setup
  src/core/tests/test_XSMeshHomogenized.cpp, 2x3_1.xml, 2x3_2.xml
                                           pin-homogenised nu-Sigma_f
and writes tests/golden/reference_known_answers.json. It also copies the
reference's own inputs that the tests run unchanged:
  examples/c5g7.xsl      the 7-group library of MOCC's tests and examples
                         (src/core/tests/c5g7.xsl and
                         src/sweepers/moc/tests/c5g7.xsl are the same file)
  examples/3x3.xml       3x3 UO2/MOX pins with a reflector, vacuum faces
  examples/c5g7_2d.xml   the 2-D quarter core of the same benchmark
into tests/golden/ under the names c5g7.xsl, example_3x3.xml and
example_c5g7_2d.xml.

Usage: python tests/golden/make_golden.py <path of a MOCC checkout>
"""
import json
import re
import sys
from pathlib import Path


def main(root):
    t = Path(root) / "src/sweepers/moc/tests"
    ray = (t / "test_Ray.cpp").read_text()
    out = {"source": "youngmit/mocc src/sweepers/moc/tests"}

    # weird_ray: inline XML, points, expected FSR ids and lengths
    m = re.search(r"TEST\(weird_ray\)(.*)", ray, re.S)
    body = m.group(1)
    xml = "".join(re.findall(r'^\s*"(.*)"\s*$', body.split("pugi::xml_document")[0], re.M))
    xml = xml.replace('\\"', '"')
    out["weird_ray"] = {
        "xml": xml,
        "p1": [-1.249999999999996 + 5.0, -5.0 + 5.0],
        "p2": [-5 + 5.0, -4.2424242424242422 + 5.0],
        "seg_index": [int(v) for v in re.findall(r"-?\d+", re.search(r"seg_index_expect = \{(.*?)\};", body, re.S).group(1))],
        "seg_len": [float(v) for v in re.findall(r"[0-9.eE+-]+", re.search(r"seg_len_expect = \{(.*?)\};", body, re.S).group(1))],
        "tol": 1e-15,
    }
    # simple_ray on 6x5.xml: the two fully asserted rays
    out["six_by_five_xml"] = (t / "6x5.xml").read_text()
    out["simple_ray"] = [
        {"p1": [0.0, 1.0], "p2": [4.0, 5.0], "cm_surf_fw": 37, "cm_cell_fw": 6, "cm_surf_bw": 88, "cm_cell_bw": 27,
         "nseg": 12, "ncseg": 8, "seg_len": (1.0 / 3.0) * 2 ** 0.5,
         "fw": ["EAST", "NORTH", "EAST", "NORTH", "EAST", "NORTH", "EAST", "NORTH"],
         "bw": ["WEST", "SOUTH", "WEST", "SOUTH", "WEST", "SOUTH", "SOUTH", "WEST"],
         "nseg_cm": [3, 0, 3, 0, 3, 0, 3, 0]},
        {"p1": [4.0, 0.0], "p2": [6.0, 2.0], "cm_surf_fw": 89, "cm_cell_fw": 4, "cm_surf_bw": 43, "cm_cell_bw": 11,
         "nseg": 6, "ncseg": 4},
    ]
    # check the transcription against the test source
    for v in ("37", "88", "89", "43"):
        assert v in ray
    out["large_xml"] = (t / "large.xml").read_text()
    out["big_ray"] = {"p1": [64.050000000000011, 0.0], "p2": [64.260000000000019, 0.024230769230770152], "ncseg": 1}
    out["square_xml"] = (t / "square.xml").read_text()
    rd = (t / "test_RayData.cpp").read_text()
    assert "0.1764 * 4.0 * PI" in rd and 'order=\\"4\\"' in rd and 'spacing=\\"0.01\\"' in rd
    out["raydata_volume"] = {"ang_quad": '<ang_quad type="ls" order="4" />', "spacing": 0.01,
                             "area_4pi": 0.1764, "tol": 1e-14}
    # XSMeshHomogenized: pin-homogenised nu-Sigma_f (group 1) of the 2x3
    # UO2/MOX lattice and of solid UO2 pins (src/core/tests)
    ct = Path(root) / "src/core/tests"
    hom = (ct / "test_XSMeshHomogenized.cpp").read_text()
    body = hom[hom.index("for (int ilat = 0; ilat < 96; ilat++)"):]
    body = body[:body.index("}")]
    pattern = [float(v) for v in re.findall(r"CHECK_CLOSE\(([0-9.eE+-]+), xs_mesh\[ilat \* 6 \+ \d\]", body)]
    solid = float(re.search(r"CHECK_CLOSE\(([0-9.eE+-]+), xs_mesh\[i\]\.xsmacnf\(0\)", hom).group(1))
    assert len(pattern) == 6
    out["xsmesh_homogenized"] = {"lattice_xml": (ct / "2x3_2.xml").read_text(),
                                 "solid_xml": (ct / "2x3_1.xml").read_text(),
                                 "nu_fission_pattern": pattern, "solid_uo2_nu_fission": solid, "tol": 1e-6}
    here = Path(__file__).resolve().parent
    dst = here / "reference_known_answers.json"
    dst.write_text(json.dumps(out, indent=1))
    print("wrote", dst)
    lib = (Path(root) / "examples/c5g7.xsl").read_bytes()
    for other in ("src/core/tests/c5g7.xsl", "src/sweepers/moc/tests/c5g7.xsl"):
        assert (Path(root) / other).read_bytes() == lib, other
    for src, name in (("examples/c5g7.xsl", "c5g7.xsl"), ("examples/3x3.xml", "example_3x3.xml"),
                      ("examples/c5g7_2d.xml", "example_c5g7_2d.xml")):
        (here / name).write_bytes((Path(root) / src).read_bytes())
        print("copied", src, "->", here / name)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit(__doc__)
    main(sys.argv[1])
