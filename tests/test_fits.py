"""FITS image output and input (gpuvmem_gb300/fits.py) on the host: the
block and card layout of the FITS standard, a round trip of image and
header values, and OCopyFITS's semantics (template header kept, BUNIT, NITER,
RADESYS, EQUINOX, CRVAL updated, plane `index` times fg_scale)."""

import numpy as np
import pytest

from gpuvmem_gb300 import fits


def _template(tmp_path):
    cards = fits.image_header(64, 64, -1.388e-5, 1.388e-5, 33.0, 33.0, ra_deg=83.63,
                              dec_deg=-30.0, freq_hz=230e9, bmaj_deg=2e-5, bmin_deg=1e-5,
                              bpa_deg=12.5)
    cards.append(("NOISE", 1.5e-4, "estimated noise"))
    cards.append(("OBJECT", "it's a test", ""))
    p = str(tmp_path / "template.fits")
    fits.write_image(p, np.zeros((64, 64), np.float32), cards)
    return p


def test_layout_and_round_trip(tmp_path):
    p = _template(tmp_path)
    raw = open(p, "rb").read()
    assert len(raw) % fits.BLOCK == 0
    assert raw[:80].decode() == f"{'SIMPLE  =                    T / conforms to FITS standard':<80}"
    assert raw[80:160].decode().startswith("BITPIX  =                  -32")
    cards, data = fits.read(p)
    assert data.shape == (64, 64) and data.dtype == np.float32
    hv = fits.header_values(p)
    assert (hv.M, hv.N, hv.bitpix) == (64, 64, -32)
    assert hv.DELTAX == -1.388e-5 and hv.crpix1 == 33.0 and hv.ra == 83.63
    assert hv.beam_bpa == 12.5 and hv.beam_noise == 1.5e-4 and hv.radesys == "ICRS"
    assert dict((k, v) for k, v, _ in cards)["OBJECT"] == "it's a test"


def test_copy_fits_semantics(tmp_path):
    p = _template(tmp_path)
    rng = np.random.default_rng(3)
    img = rng.normal(0, 1, (2, 64, 64)).astype(np.float32)
    out = str(tmp_path / "mem.fits")
    fits.copy_fits(img, p, out, units="JY/PIXEL", iteration=17, index=1, fg_scale=3e-4,
                   ra_center=84.0, frame="FK5", equinox=1950.0)
    cards, data = fits.read(out)
    kv = {k: v for k, v, _ in cards}
    assert kv["NITER"] == 17 and kv["BUNIT"] == "JY/PIXEL" and kv["RADESYS"] == "FK5"
    assert kv["EQUINOX"] == 1950.0 and kv["CRVAL1"] == 84.0 and kv["CRVAL2"] == -30.0
    assert kv["BMAJ"] == 2e-5 and kv["NOISE"] == 1.5e-4  # the template's other cards
    np.testing.assert_array_equal(data, img[1] * np.float32(3e-4))
    np.testing.assert_array_equal(fits.read_image(out), img[1] * np.float32(3e-4))


def test_missing_required_key(tmp_path):
    p = str(tmp_path / "bad.fits")
    fits.write_image(p, np.zeros((8, 8), np.float32), [("CDELT1", -1e-5, "")])
    with pytest.raises(ValueError):
        fits.header_values(p)


def test_card_formatting():
    c = fits.format_card("CRVAL1", 83.63, "ra")
    assert len(c) == 80 and c[8:10] == "= " and c[10:30].strip() == "83.63"
    assert fits.format_card("OBJECT", "x").startswith("OBJECT  = 'x       '")
    assert fits._parse_value("'O''Brien'  / who") == ("O'Brien", "who")
    assert fits._parse_value("  1.5D-3 / d exponent")[0] == 1.5e-3
