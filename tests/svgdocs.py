"""Seeded SVG documents for the front-end tests: groups with transforms,
fills and strokes of every cap and join, gradients, a clip path, every
path-data command."""
import numpy as np

CAPS = ("butt", "round", "square")
JOINS = ("miter", "round", "bevel")


def random_path_data(rng, cx, cy, r):
    k = int(rng.integers(3, 8))
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    pts = [(cx + r * rng.uniform(0.4, 1) * np.cos(a), cy + r * rng.uniform(0.4, 1) * np.sin(a)) for a in ang]
    d = [f"M{pts[0][0]:.3f} {pts[0][1]:.3f}"]
    for i in range(1, k):
        x, y = pts[i]
        px, py = pts[i - 1]
        c = rng.integers(0, 6)
        if c == 0:
            d.append(f"L{x:.3f} {y:.3f}")
        elif c == 1:
            d.append(f"c{(x - px) / 3 + rng.normal(0, 4):.3f} {(y - py) / 3:.3f} "
                     f"{2 * (x - px) / 3:.3f} {2 * (y - py) / 3 + rng.normal(0, 4):.3f} {x - px:.3f} {y - py:.3f}")
        elif c == 2:
            d.append(f"Q{(px + x) / 2 + rng.normal(0, 5):.3f} {(py + y) / 2:.3f} {x:.3f} {y:.3f}")
        elif c == 3:
            d.append(f"S{x + rng.normal(0, 4):.3f} {y:.3f} {x:.3f} {y:.3f}")
        elif c == 4:
            d.append(f"A{r / 2:.3f} {r / 3:.3f} {rng.uniform(0, 90):.1f} 0 1 {x:.3f} {y:.3f}")
        else:
            d.append(f"H{x:.3f}V{y:.3f}")
    if rng.integers(0, 2):
        d.append("Z")
    return " ".join(d)


def document(seed=0, n=24, W=256, H=192):
    rng = np.random.default_rng(seed)
    out = [f'<svg xmlns="http://www.w3.org/2000/svg" width="{W}" height="{H}" viewBox="0 0 {W / 2} {H / 2}">',
           '<defs><linearGradient id="lg" x1="0" y1="0" x2="1" y2="1"><stop offset="0" stop-color="#e04"/>'
           '<stop offset="1" stop-color="#04e" stop-opacity="0.6"/></linearGradient>'
           '<radialGradient id="rg" spreadMethod="reflect"><stop offset="0.2" stop-color="yellow"/>'
           '<stop offset="1" stop-color="green"/></radialGradient>'
           f'<clipPath id="cp"><circle cx="{W / 4}" cy="{H / 4}" r="{min(W, H) / 5}"/></clipPath></defs>']
    for i in range(n):
        tr = f'translate({rng.uniform(-10, 10):.2f},{rng.uniform(-10, 10):.2f}) rotate({rng.uniform(-30, 30):.1f})'
        fill = rng.choice(["none", "url(#lg)", "url(#rg)", f"#{int(rng.integers(0, 0xffffff)):06x}"])
        sw = float(rng.choice([0.01, 0.5, 1.5, 3.0]))
        attrs = (f'fill="{fill}" stroke="#{int(rng.integers(0, 0xffffff)):06x}" stroke-width="{sw}" '
                 f'stroke-linecap="{CAPS[i % 3]}" stroke-linejoin="{JOINS[(i // 3) % 3]}" '
                 f'stroke-opacity="{rng.uniform(0.5, 1):.2f}"')
        clip = ' clip-path="url(#cp)"' if i % 7 == 3 else ""
        out.append(f'<g transform="{tr}"{clip}><path d="{random_path_data(rng, rng.uniform(10, W / 2 - 10), rng.uniform(10, H / 2 - 10), rng.uniform(5, 30))}" {attrs}/></g>')
    out.append('<rect x="5" y="5" width="20" height="12" rx="3" fill="none" stroke="black" stroke-width="1"/>')
    out.append('<polyline points="30,5 40,15 50,5 60,15" fill="none" stroke="#333" stroke-width="2" '
               'stroke-linejoin="round" stroke-linecap="round"/>')
    out.append("</svg>")
    return "\n".join(out)
