"""The oracle against the reference's own known-answer tests (oracle/kat.cpp
restates them; each case names the Go test it comes from)."""
import subprocess

import pytest


@pytest.fixture(scope="module")
def kat_results(oracle):
    out = subprocess.run([oracle.KAT], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, timeout=300)
    lines = out.stdout.decode().splitlines()
    return out.returncode, lines


def test_kat_all_pass(kat_results):
    rc, lines = kat_results
    fails = [l for l in lines if l.startswith("FAIL")]
    assert rc == 0 and not fails, "\n".join(fails)
    summary = [l for l in lines if l.startswith("SUMMARY")][0]
    npass = int(summary.split("pass=")[1].split()[0])
    assert npass >= 138


@pytest.mark.parametrize("family", [
    "TestCalculateMISWeight", "TestPdfPropagation", "TestLightPathBetaPropagation",
    "TestCameraPathBetaPropagation", "TestEvaluateDirectLightingStrategy", "TestVertexConvertSolidAngleToAreaPdf",
    "TestTriangle_Hit", "TestQuad_Hit", "TestSphere_Hit", "TestBox_Hit", "TestWorldRadius", "TestWeFunction",
    "TestMapRayToPixel", "TestPowerHeuristic", "TestDielectricEvaluateBRDF",
    "TestDiscHit", "TestCylinder_Hit_SimpleHit", "TestCylinder_Capped_HitTopCap", "TestCylinder_Hit_ArbitraryOrientation",
    "TestCone_Hit_Frustum", "TestCone_Capped_HitBaseCap_Pointed", "TestCone_Uncapped_NoCapHits",
    "TestPointSpotLight_PDF", "TestDiscLightPDF", "TestDiscSpotLightFalloff", "TestImageTextureEvaluate",
    "TestImageTextureWrapping",
])
def test_kat_family_present_and_passing(kat_results, family):
    _, lines = kat_results
    mine = [l for l in lines if family in l]
    assert mine, "no cases for " + family
    assert all(l.startswith("PASS") for l in mine), "\n".join(mine)
