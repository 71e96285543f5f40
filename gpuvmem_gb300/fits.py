"""FITS image input and output for the imaging path, written from the FITS
standard (version 4.0: 2880-byte blocks, 80-character header cards,
big-endian data) without cfitsio.

  header_values(path)   readFITSHeader (src/MSFITSIO.cu:318-380): the
                        header values the reference reads from its model
                        input (CDELT, CRVAL, CRPIX, NAXIS, BMAJ/BMIN/BPA,
                        NOISE, RADESYS, EQUINOX, BITPIX)
  read_image(path)      the primary image as float32 [NAXIS2, NAXIS1]
  write_image(...)      a primary HDU from header cards and an image
  copy_fits(...)        OCopyFITS (src/MSFITSIO.cu:94-168): the template's
                        header with BUNIT, NITER, NAXIS1/2, RADESYS, EQUINOX,
                        CRVAL1/2 updated, and plane `index` of the image
                        times fg_scale as the data
  image_header(...)     a header for a run without a template (synthetic
                        data): SIN projection at the phase centre

Values are kept as Python types: str, bool, int, float.  Host code only (the
image is copied from the device when it is a CUDA tensor).
"""

from __future__ import annotations

import dataclasses
from typing import Dict, List, Optional, Sequence, Tuple, Union

import numpy as np

BLOCK = 2880
CARD = 80
_BITPIX = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}

Card = Tuple[str, object, str]  # keyword, value (None for commentary cards), comment


# ------------------------------------------------------------------ cards
def _format_value(v) -> str:
    if isinstance(v, bool):
        return f"{'T' if v else 'F':>20}"
    if isinstance(v, (int, np.integer)):
        return f"{int(v):>20d}"
    if isinstance(v, (float, np.floating)):
        s = repr(float(v)).upper()
        if "E" not in s and "." not in s and "INF" not in s and "NAN" not in s:
            s += ".0"
        if len(s) > 20:
            s = f"{float(v):.13E}"
        return f"{s:>20}"
    s = str(v).replace("'", "''")
    return f"'{s:<8}'"


def format_card(key: str, value=None, comment: str = "") -> str:
    """One 80-character header card (fixed format)."""
    key = key.upper()
    if len(key) > 8:
        raise ValueError(f"keyword {key!r} longer than 8 characters")
    if key in ("COMMENT", "HISTORY", "") or value is None:
        text = f"{key:<8}{comment}" if key else f"        {comment}"
    else:
        text = f"{key:<8}= {_format_value(value)}"
        if comment:
            text += f" / {comment}"
    if len(text) > CARD:
        text = text[:CARD]
    return f"{text:<{CARD}}"


def _parse_value(s: str):
    s = s.strip()
    if not s:
        return None, ""
    if s.startswith("'"):
        out, i = [], 1
        while i < len(s):
            if s[i] == "'":
                if i + 1 < len(s) and s[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(s[i])
            i += 1
        rest = s[i + 1:]
        com = rest.split("/", 1)[1].strip() if "/" in rest else ""
        return "".join(out).rstrip(), com
    val, com = (s.split("/", 1) + [""])[:2]
    val = val.strip()
    if val in ("T", "F"):
        return val == "T", com.strip()
    try:
        return int(val), com.strip()
    except ValueError:
        pass
    try:
        return float(val.replace("D", "E")), com.strip()
    except ValueError:
        return val, com.strip()


def parse_cards(raw: bytes) -> Tuple[List[Card], int]:
    """Cards of one header and the number of bytes the header occupies."""
    cards: List[Card] = []
    pos = 0
    while True:
        if pos + CARD > len(raw):
            raise ValueError("FITS header without END")
        text = raw[pos:pos + CARD].decode("ascii", errors="replace")
        pos += CARD
        key = text[:8].strip()
        if key == "END":
            break
        if text[8:10] == "= ":
            v, c = _parse_value(text[10:])
            cards.append((key, v, c))
        else:
            cards.append((key, None, text[8:].rstrip()))
    return cards, ((pos + BLOCK - 1) // BLOCK) * BLOCK


def header_bytes(cards: Sequence[Card]) -> bytes:
    text = "".join(format_card(k, v, c) for k, v, c in cards) + format_card("END")
    text += " " * ((-len(text)) % BLOCK)
    return text.encode("ascii")


def _get(cards: Sequence[Card], key: str, default=None):
    for k, v, _ in cards:
        if k == key and v is not None:
            return v
    return default


def update_key(cards: List[Card], key: str, value, comment: Optional[str] = None) -> None:
    """fits_update_key: replace the value (and comment, if given) of `key`,
    or append the card."""
    for i, (k, v, c) in enumerate(cards):
        if k == key and v is not None:
            cards[i] = (k, value, c if comment is None else comment)
            return
    cards.append((key, value, comment or ""))


# ------------------------------------------------------------------ files
def read(path: str) -> Tuple[List[Card], np.ndarray]:
    """Primary header cards and data (native byte order, FITS axis order
    reversed: [NAXISn, ..., NAXIS1]), with BSCALE/BZERO applied."""
    raw = open(path, "rb").read()
    cards, hlen = parse_cards(raw)
    if _get(cards, "SIMPLE") is not True:
        raise ValueError(f"{path}: not a FITS file (SIMPLE != T)")
    bitpix = int(_get(cards, "BITPIX"))
    naxis = int(_get(cards, "NAXIS", 0))
    shape = tuple(int(_get(cards, f"NAXIS{i}")) for i in range(naxis, 0, -1))
    count = int(np.prod(shape)) if naxis else 0
    data = np.frombuffer(raw, dtype=_BITPIX[bitpix], count=count, offset=hlen).reshape(shape)
    bscale, bzero = float(_get(cards, "BSCALE", 1.0)), float(_get(cards, "BZERO", 0.0))
    data = data.astype(np.float64 if bitpix in (-64, 32, 64) else np.float32)
    if bscale != 1.0 or bzero != 0.0:
        data = data * bscale + bzero
    return cards, data


def read_image(path: str) -> np.ndarray:
    """The primary image as float32 [NAXIS2, NAXIS1] (degenerate axes such
    as Stokes and frequency dropped)."""
    _, data = read(path)
    img = np.asarray(data, dtype=np.float32)
    while img.ndim > 2 and img.shape[0] == 1:
        img = img[0]
    return img


def write_image(path: str, image: np.ndarray, cards: Optional[Sequence[Card]] = None,
                bitpix: int = -32) -> None:
    """A primary HDU: the structural cards (SIMPLE, BITPIX, NAXISn, EXTEND)
    followed by the other cards of `cards`, then the image in big-endian
    order, padded to the 2880-byte block."""
    image = np.asarray(image)
    if bitpix not in (-32, -64):
        raise ValueError("only floating-point images are written (BITPIX -32 or -64)")
    out: List[Card] = [("SIMPLE", True, "conforms to FITS standard"),
                       ("BITPIX", bitpix, "array data type"),
                       ("NAXIS", image.ndim, "number of array dimensions")]
    for i, n in enumerate(image.shape[::-1], start=1):
        out.append((f"NAXIS{i}", int(n), ""))
    out.append(("EXTEND", True, ""))
    skip = {"SIMPLE", "BITPIX", "NAXIS", "EXTEND", "END", "BSCALE", "BZERO"}
    for k, v, c in cards or []:
        if k in skip or (k.startswith("NAXIS") and k[5:].isdigit()):
            continue
        out.append((k, v, c))
    body = np.ascontiguousarray(image, dtype=_BITPIX[bitpix]).tobytes()
    body += b"\0" * ((-len(body)) % BLOCK)
    with open(path, "wb") as f:
        f.write(header_bytes(out))
        f.write(body)


@dataclasses.dataclass
class HeaderValues:
    """headerValues of the reference (include/MSFITSIO.cuh:140-156)."""
    DELTAX: float
    DELTAY: float
    ra: float
    dec: float
    crpix1: float
    crpix2: float
    M: int
    N: int
    beam_bmaj: float
    beam_bmin: float
    beam_bpa: float
    beam_noise: float
    radesys: str
    equinox: float
    bitpix: int


def header_values(path: str) -> HeaderValues:
    """readFITSHeader (src/MSFITSIO.cu:318-380).  CDELT1/2, CRVAL1/2,
    CRPIX1/2, NAXIS1/2 and RADESYS are required (the reference exits without
    them; here ValueError); a missing NOISE reads as -1 and EQUINOX as 2000,
    as there; a missing BMAJ/BMIN/BPA (left unset by the reference) as 0."""
    cards, _ = parse_cards(open(path, "rb").read(BLOCK * 64))
    for key in ("CDELT1", "CDELT2", "CRVAL1", "CRVAL2", "CRPIX1", "CRPIX2", "NAXIS1", "NAXIS2",
                "RADESYS"):
        if _get(cards, key) is None:
            raise ValueError(f"{path}: header keyword {key} is missing")
    g = lambda k, d=None: _get(cards, k, d)  # noqa: E731
    return HeaderValues(float(g("CDELT1")), float(g("CDELT2")), float(g("CRVAL1")),
                        float(g("CRVAL2")), float(g("CRPIX1")), float(g("CRPIX2")),
                        int(g("NAXIS1")), int(g("NAXIS2")), float(g("BMAJ", 0.0)),
                        float(g("BMIN", 0.0)), float(g("BPA", 0.0)), float(g("NOISE", -1.0)),
                        str(g("RADESYS", "ICRS")), float(g("EQUINOX", 2000.0)),
                        int(g("BITPIX")))


def image_header(M: int, N: int, deltax_deg: float, deltay_deg: float, crpix1: float,
                 crpix2: float, ra_deg: float = 0.0, dec_deg: float = 0.0,
                 freq_hz: Optional[float] = None, bmaj_deg: float = 0.0, bmin_deg: float = 0.0,
                 bpa_deg: float = 0.0, radesys: str = "ICRS",
                 equinox: float = 2000.0) -> List[Card]:
    """Header cards of an image with no template (SIN projection)."""
    cards: List[Card] = [
        ("BUNIT", "JY/PIXEL", "Unit of measurement"),
        ("CTYPE1", "RA---SIN", ""), ("CRVAL1", float(ra_deg), ""),
        ("CDELT1", float(deltax_deg), ""), ("CRPIX1", float(crpix1), ""),
        ("CUNIT1", "deg", ""),
        ("CTYPE2", "DEC--SIN", ""), ("CRVAL2", float(dec_deg), ""),
        ("CDELT2", float(deltay_deg), ""), ("CRPIX2", float(crpix2), ""),
        ("CUNIT2", "deg", ""),
        ("BMAJ", float(bmaj_deg), ""), ("BMIN", float(bmin_deg), ""),
        ("BPA", float(bpa_deg), ""),
        ("RADESYS", radesys, ""), ("EQUINOX", float(equinox), "")]
    if freq_hz is not None:
        cards += [("RESTFRQ", float(freq_hz), "")]
    return cards


def copy_fits(image, template: Union[str, Sequence[Card]], path: str, units: str = "JY/PIXEL",
              iteration: int = 0, index: int = 0, fg_scale: float = 1.0,
              ra_center: Optional[float] = None, dec_center: Optional[float] = None,
              frame: Optional[str] = None, equinox: Optional[float] = None) -> None:
    """OCopyFITS (src/MSFITSIO.cu:94-168): plane `index` of the image (host
    array or CUDA tensor of P x N x M values) times fg_scale, under the
    template's header with BUNIT, NITER, NAXIS1, NAXIS2, RADESYS, EQUINOX,
    CRVAL1 and CRVAL2 updated (the last four keep the template's values
    where not given)."""
    if hasattr(image, "detach"):
        image = image.detach().cpu().numpy()
    img = np.asarray(image, dtype=np.float32)
    plane = img.reshape(-1, img.shape[-2], img.shape[-1])[index]
    N, M = plane.shape
    if isinstance(template, str):
        cards = list(parse_cards(open(template, "rb").read())[0])
    else:
        cards = list(template)
    update_key(cards, "BUNIT", units, "Unit of measurement")
    update_key(cards, "NITER", int(iteration), "Number of iteration in gpuvmem software")
    if frame is not None:
        update_key(cards, "RADESYS", frame, "Changed by gpuvmem")
    if equinox is not None:
        update_key(cards, "EQUINOX", float(equinox), "Changed by gpuvmem")
    if ra_center is not None:
        update_key(cards, "CRVAL1", float(ra_center), "Changed by gpuvmem")
    if dec_center is not None:
        update_key(cards, "CRVAL2", float(dec_center), "Changed by gpuvmem")
    # host_IFITS[N*i + j] *= fg_scale, in FP32
    data = (plane * np.float32(fg_scale)).astype(np.float32)
    write_image(path, data, cards, bitpix=-32)
