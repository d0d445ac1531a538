"""The eFacetEB process entry's host parts (no GPU): the XML reading of
runFacetEBCore (firstXmlTag, xmlFloat: facetrtcore.cpp:2068-2110), the
spectrum reader (readScalarSpectrum :2499-2509) and the error paths that
come before any device work."""
import numpy as np
import pytest

from streamsim_gb300 import faceteb


def test_first_xml_tag_and_xml_float():
    xml = ('<A><dTime>900</dTime><dTime>60</dTime><Latitude unit="deg"> 31.5 </Latitude>'
           '<x>1.5abc</x><y>abc</y><z>inf</z><w>&lt;7&gt;</w><e>2e3</e><n></n></A>')
    assert faceteb.first_xml_tag(xml, "dTime") == "900"  # the first one
    assert faceteb.first_xml_tag(xml, "w") == "<7>"      # entities decoded
    assert faceteb.first_xml_tag(xml, "missing") == ""
    assert faceteb.xml_float(xml, "Latitude", 40.0) == 31.5  # attributes, spaces
    assert faceteb.xml_float(xml, "x", 0.0) == 1.5            # stof's number prefix
    assert faceteb.xml_float(xml, "y", 7.0) == 7.0            # unparsable: fallback
    assert faceteb.xml_float(xml, "z", 7.0) == 7.0            # not finite: fallback
    assert faceteb.xml_float(xml, "n", 3.0) == 3.0            # empty: fallback
    assert faceteb.xml_float(xml, "e", 0.0) == 2000.0
    assert faceteb.xml_float("<a>0.1</a>", "a", 0.0) == float(np.float32(0.1))


def test_scalar_spectrum(tmp_path):
    p = tmp_path / "esun.dat"
    p.write_text("1.5 -2\n3 nan 4 x 5\n")
    assert faceteb._scalar_spectrum(str(p)).tolist() == [1.5, 0.0, 3.0, 0.0, 4.0]
    p.write_text(" ".join(["1"] * 2100))
    assert faceteb._scalar_spectrum(str(p)).size == 2001
    assert faceteb._scalar_spectrum(str(tmp_path / "none.dat")).size == 0


def test_missing_meteorology_and_short_tables(tmp_path):
    xml = tmp_path / "Input.xml"
    xml.write_text("<HiStreamProject><Meteorology><filePath>met/none.txt</filePath>"
                   "</Meteorology></HiStreamProject>")
    with pytest.raises(RuntimeError, match="^FacetEB cannot open meteorology: met/none.txt$"):
        faceteb.run_faceteb_core(str(xml), str(tmp_path / "out" / "faceteb.json"), progress=None)
    (tmp_path / "met.txt").write_text("header\n1.5 20 15 1000 2 300 330\n")
    xml.write_text("<HiStreamProject><filePath>met.txt</filePath><endTimeNode>3</endTimeNode>"
                   "</HiStreamProject>")
    with pytest.raises(RuntimeError, match="^FacetEB time range exceeds meteorology rows$"):
        faceteb.run_faceteb_core(str(xml), "", progress=None)
    assert faceteb.main([]) == 2
