//! Renders a textured unit cube the way the reference demo drives its Renderer
//! (src/main.rs:129-184 of the reference crate) and writes the frame as a binary PPM.
use rusterizer_gb300::*;

fn checkerboard(n: usize, square: usize) -> Texture {
    let mut buf = Vec::with_capacity(n * n * 4);
    for y in 0..n {
        for x in 0..n {
            let v = if ((x / square) + (y / square)) % 2 == 0 { 255 } else { 128 };
            buf.extend_from_slice(&[v, v, v, 255]);
        }
    }
    Texture::from_rgba8(buf, n, n)
}

fn cube() -> Mesh {
    // six faces, four vertices each, uvs (0,0) (1,0) (1,1) (0,1)
    let faces: [([f32; 3], [f32; 3], [f32; 3]); 6] = [
        ([0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]),
        ([0.0, 0.0, -1.0], [-1.0, 0.0, 0.0], [0.0, 1.0, 0.0]),
        ([1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]),
        ([-1.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, 1.0, 0.0]),
        ([0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, -1.0]),
        ([0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]),
    ];
    let mut m = Mesh::default();
    for (n, u, v) in faces {
        let base = m.vertices.len();
        for (su, sv, uv) in [(-1.0, 1.0, [0.0, 0.0]), (1.0, 1.0, [1.0, 0.0]), (1.0, -1.0, [1.0, 1.0]), (-1.0, -1.0, [0.0, 1.0])] {
            let p = [0, 1, 2].map(|k| 0.5 * (n[k] + su * u[k] + sv * v[k]));
            m.vertices.push(p);
            m.attributes.push((Color::new(1.0, 1.0, 1.0, 1.0), uv).into());
        }
        m.indices.extend_from_slice(&[base, base + 1, base + 2, base, base + 2, base + 3]);
    }
    m
}

fn perspective(near: f32, far: f32, aspect: f32, fov: f32) -> Mat4 {
    let hw = (fov / 2.0).tan() * near;
    let hh = aspect * hw;
    [
        [near / hw, 0.0, 0.0, 0.0],
        [0.0, near / hh, 0.0, 0.0],
        [0.0, 0.0, -(far + near) / (far - near), -2.0 * far * near / (far - near)],
        [0.0, 0.0, -1.0, 0.0],
    ]
}

fn main() {
    let (w, h) = (800usize, 600usize);
    let mut r = Renderer::new(w, h);
    r.uniforms().bind_texture(0, checkerboard(64, 8));
    let mesh = cube();
    let (s, c) = (0.5f32.sin(), 0.5f32.cos());
    let blk = r.uniforms().write_block();
    blk.world = [[c, 0.0, s, 0.0], [0.0, 1.0, 0.0, 0.0], [-s, 0.0, c, -3.0], [0.0, 0.0, 0.0, 1.0]];
    blk.view = identity();
    blk.projection = perspective(0.1, 100.0, h as f32 / w as f32, std::f32::consts::FRAC_PI_3);
    r.render(&mesh, MvpVertexShader, TextureShader);
    let fb = r.framebuffer().to_vec();
    let mut ppm = format!("P6 {} {} 255\n", w, h).into_bytes();
    for p in fb {
        ppm.extend_from_slice(&[(p >> 16) as u8, (p >> 8) as u8, p as u8]);
    }
    std::fs::write("cube.ppm", ppm).expect("write cube.ppm");
    println!("wrote cube.ppm; stats {:?}", r.stats());
}
