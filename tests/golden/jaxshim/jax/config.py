class _Config:
    def update(self, *args, **kwargs):
        pass


config = _Config()
