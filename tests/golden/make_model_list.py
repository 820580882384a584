"""Write ``model_list.json``: each model string the reference's
``ac::specs::ModelList`` lists (core/include/AC/Specs.hpp) with its stated
parameter count and, for third-party models, version, author and homepage,
read from the header as text.  The tests compare ``pyac.specs.ModelList``
against it.

Usage: python tests/golden/make_model_list.py [path to the Anime4KCPP sources]
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AC_REFERENCE_ROOT", "")
if not SRC:
    sys.exit("usage: %s REFERENCE_ROOT (or set AC_REFERENCE_ROOT)" % sys.argv[0])

text = open(os.path.join(SRC, "core", "include", "AC", "Specs.hpp")).read()
models = []
for m in re.finditer(r'\{\s*"([a-z0-9-]+)",\s*"[^"]*",\s*(\d+)(?:,\s*"([^"]*)",\s*"([^"]*)",\s*"([^"]*)")?', text):
    models.append({"name": m.group(1), "parameter_count": int(m.group(2)),
                   "version": m.group(3), "author": m.group(4), "homepage": m.group(5)})
with open(os.path.join(HERE, "model_list.json"), "w") as f:
    json.dump(models, f, indent=1)
    f.write("\n")
print(len(models), "models")
