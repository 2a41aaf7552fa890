{
  "targets": [
    {
      "target_name": "avbd_node",
      "sources": ["avbd_node.cc"],
      "include_dirs": ["../../include"],
      "cflags_cc": ["-std=c++17", "-O2"],
      "libraries": ["-L<(module_root_dir)/..", "-lavbd_gb300", "-Wl,-rpath,<(module_root_dir)/.."]
    }
  ]
}
