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
    import json
    index = json.loads((tmp_path / "out" / "faceteb_run.json").read_text())
    assert index["status"] == "failed" and index["kind"] == "faceteb-run"
    assert index["requested"] == {"endNodeExclusive": 1, "startNode": 0}
    assert list(index) == sorted(index) and "finishedAt" in index
    (tmp_path / "met.txt").write_text("header\n1.5 20 15 1000 2 300 330\n")
    xml.write_text("<HiStreamProject><filePath>met.txt</filePath><endTimeNode>3</endTimeNode>"
                   "</HiStreamProject>")
    with pytest.raises(RuntimeError, match="^FacetEB time range exceeds meteorology rows$"):
        faceteb.run_faceteb_core(str(xml), "", progress=None)
    assert faceteb.main([]) == 2


def test_photovoltaic_tables(tmp_path):
    """photovoltaic_node_<node>.csv and photovoltaic_summary.csv
    (facetrtcore.cpp:3847-3860) from one node's fields: PV facets only,
    front-side values, area-weighted sums, the energy running over nodes."""
    from streamsim_gb300 import facetcu
    F, leaf = 4, 3
    v = np.zeros((3 * F, 6), np.float32)
    for f in range(F):  # right triangles of legs 1 and f + 1: area (f + 1) / 2
        v[3 * f + 1, 0] = 1.0
        v[3 * f + 2, 2] = f + 1.0
    assert np.array_equal(faceteb.facet_areas(v), np.float32([0.5, 1.0, 1.5, 2.0]))
    mats = [facetcu.EnergySurface(), facetcu.EnergySurface(photovoltaic=True, pv_bifaciality=0.25)]

    class Model:
        facet_count = F

        def computeSunlitFraction(self, sun):  # not called here
            raise AssertionError

    run = faceteb.Run(Model(), leaf, mats, np.array([1, 0, 1, 0], np.uint32), time_step=3600.0)
    S = 2 * F
    fields = {k: np.arange(S, dtype=np.float32) + 1 for k in
              ("absorbed_shortwave", "incident_shortwave", "photovoltaic_power", "net_radiation",
               "sensible_heat", "latent_heat", "storage_heat")}
    fields["temperature"] = np.full(S, 300.0, np.float32)
    with open(tmp_path / "photovoltaic_summary.csv", "w") as summary:
        summary.write(faceteb.PV_SUMMARY_HEADER)
        e, pa = run._write_pv(str(tmp_path), 0, "DOY1_00-00", fields, faceteb.facet_areas(v),
                              run._pv_facets(), summary, 0.0)
        assert pa == 2.0  # PV facets 0 and 2: 0.5 + 1.5
        e, _ = run._write_pv(str(tmp_path), 1, "DOY1_01-00", fields, faceteb.facet_areas(v),
                             run._pv_facets(), summary, e)
    rows = (tmp_path / "photovoltaic_node_0.csv").read_text().splitlines()
    assert rows[0] == faceteb.PV_NODE_HEADER.strip() and len(rows) == 3  # facets 0 and 2
    first = rows[1].split(",")
    # facet 0: area 0.5, 26.85 C, incident 1 + 2, absorbed 3, power 1, net - absorbed
    assert first[:5] == ["0.5", "26.85", "3", "3", "1"] and first[-1] == "0"
    assert first[5] == "-3" and first[7] == "1.5"  # residual 1-1-1-1-1; 1 + 0.25 * 2
    assert first[8] == "-2"  # net longwave: net - absorbed
    summ = (tmp_path / "photovoltaic_summary.csv").read_text().splitlines()
    assert len(summ) == 3 and summ[1].split(",")[:3] == ["0", "DOY1_00-00", "2"]
    # electric power: 0.5 * 1 + 1.5 * 5 = 8 W per node; 3600 s each
    assert summ[1].split(",")[6] == "8" and summ[2].split(",")[-1] == faceteb._g(2 * 8 / 1000.0)
