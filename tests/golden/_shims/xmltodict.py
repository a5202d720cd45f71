"""Minimal stand-in for the ``xmltodict`` package (absent in this container),
enough for the reference's UPF reader (``functional/pseudo/upf.py:121-132``)
to run during golden-fixture generation.  Project-written on
``xml.etree``: an element becomes a dict of its attributes (``attr_prefix``
prepended), its children (repeated tags -> list) and ``#text``; an element
with text only becomes that text; whitespace is stripped.
"""
import xml.etree.ElementTree as ET


def _conv(el, prefix):
    d = {}
    for k, v in el.attrib.items():
        d[prefix + k] = v
    for ch in el:
        v = _conv(ch, prefix)
        if ch.tag in d:
            if not isinstance(d[ch.tag], list):
                d[ch.tag] = [d[ch.tag]]
            d[ch.tag].append(v)
        else:
            d[ch.tag] = v
    text = (el.text or "").strip()
    if not d:
        return text if text else None
    if text:
        d["#text"] = text
    return d


def parse(string, attr_prefix="@", **kwargs):
    root = ET.fromstring(string)
    return {root.tag: _conv(root, attr_prefix)}
